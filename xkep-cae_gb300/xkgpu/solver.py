"""The reference's dynamic contact solver loop over the device assembly.

``ContactFrictionSolver.run`` is ``ContactFrictionProcess.process``
(``xkep_cae/contact/solver/process.py:139-674``) with its inner
``NewtonDynamicProcess`` (``contact/solver/_newton_dynamic.py:115-398``), the
same step control, convergence tests, divergence detection, line search and
cutbacks, over an assembly backend:

* per increment: Generalized-alpha prediction, prescribed displacements
  ``u[dofs] = load_frac * values``, detection (broadphase, pair merge) and the
  geometry update with the active-set update at ``X + u``
  (``process.py:406-429``);
* per Newton attempt (``_newton_dynamic.py:160-395``): the assembly of
  ``R = f_int + f_c - f_ext`` with ``R[fixed] = 0`` (``_newton_steps.py:79-135``),
  the effective residual, the force test ``||R|| / f_ref < tol_force``
  (``_newton_steps.py:182-243``) with ``f_ref`` the first attempt's residual
  norm when there is no external load, the divergence tests, the tangent
  ``K_beam + K_c`` plus the mass term, the linear solve with the Dirichlet
  rows and columns replaced by the identity (``_newton_steps.py:338-366``),
  the line search on the internal force only (``contact/solver/_utils.py:31-61``,
  called with ``diverge_factor = 3``, ``_newton_steps.py:405-437``), the
  update and the displacement and energy tests;
* per increment result: the adaptive step control of
  ``UnifiedTimeStepProcess`` / ``AdaptiveSteppingProcess``
  (``_unified_time_controller.py:98-215``, ``_adaptive_stepping.py:73-197``):
  growth on few attempts, shrink on many or on a change of the active count,
  cutback with a retry from the last converged state on failure (the pair
  state is not rolled back, as in the reference, ``_solver_state.py:58-75``).

The backend (``EngineBackend`` for the GPU engine) supplies detection,
assembly, the internal force alone, the active count and the linear solve.
Vectors are torch tensors on the backend's device; the norms, the step
control and every decision are FP64.  Nothing here is specific to the mixed or
FP64 engine: both run the same loop.
"""

from __future__ import annotations

import math
from collections import deque
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla
import torch

from . import _lib as L
from .device import ptr, stream_handle


# --------------------------------------------------------------------------- step control


class StepControl:
    """Adaptive load-fraction control: ``UnifiedTimeStepProcess`` over ``AdaptiveSteppingProcess``.

    ``query(load_frac_prev)`` gives the next load fraction and its time
    increment, ``success(...)`` and ``failure(...)`` consume it
    (``_adaptive_stepping.py:118-197``, ``_unified_time_controller.py:160-198``).
    """

    def __init__(self, t_total: float, dt_initial: float = 0.0, dt_min: float = 0.0, dt_max: float = 0.0,
                 grow: float = 1.5, shrink: float = 0.5, grow_attempts: int = 5, shrink_attempts: int = 15,
                 contact_change: float = 0.3):
        if not t_total > 0.0:
            raise ValueError(f"t_total must be positive: {t_total}")
        # UnifiedTimeStepInput.__post_init__ (_unified_time_controller.py:66-75)
        if dt_initial <= 0.0:
            dt_initial = t_total / 20.0
        if dt_min <= 0.0:
            dt_min = dt_initial / 32.0
        if dt_max <= 0.0:
            dt_max = min(dt_initial * 4.0, t_total)
        self.t_total = t_total
        init_frac, min_frac, max_frac = dt_initial / t_total, dt_min / t_total, dt_max / t_total
        # AdaptiveSteppingInput.__post_init__ (_adaptive_stepping.py:30-39)
        eff_n = max(1, int(1.0 / init_frac) if init_frac > 0 else 1)
        if min_frac <= 0.0:
            min_frac = 1.0 / (eff_n * 32)
        if max_frac <= 0.0:
            max_frac = min(8.0 / eff_n, 1.0)
        self.grow, self.shrink = grow, shrink
        self.grow_attempts, self.shrink_attempts = grow_attempts, shrink_attempts
        self.contact_change = contact_change
        self.min_frac, self.max_frac = min_frac, max_frac
        base = init_frac if init_frac > 0.0 else 1.0
        if max_frac > 0.0:
            base = min(base, max_frac)
        self.queue: deque[float] = deque([min(base, 1.0)])
        self.consecutive_good = 0
        self.n_cutbacks = 0
        self._last_prev = 0.0

    def query(self, load_frac_prev: float) -> tuple[bool, float, float]:
        """(has more steps, load fraction, time increment of the step)."""
        while self.queue:
            nxt = self.queue[0]
            if nxt <= load_frac_prev + 1e-15:
                self.queue.popleft()
                continue
            return True, nxt, max((nxt - self._last_prev) * self.t_total, 0.0)
        return False, 0.0, max((0.0 - self._last_prev) * self.t_total, 0.0)

    def success(self, load_frac: float, load_frac_prev: float, n_attempts: int, n_active: int,
                prev_n_active: int) -> None:
        self._last_prev = load_frac
        if self.queue and self.queue[0] <= load_frac + 1e-15:
            self.queue.popleft()
        if load_frac >= 1.0 - 1e-12:
            return
        current = load_frac - load_frac_prev
        nxt = current
        if n_attempts <= self.grow_attempts:
            self.consecutive_good += 1
            if self.consecutive_good <= 2:
                nxt = current * self.grow
            else:
                damp = max(0.1, 1.0 / self.consecutive_good)
                nxt = current * (1.0 + (self.grow - 1.0) * damp)
        elif n_attempts >= self.shrink_attempts:
            nxt = current * self.shrink
            self.consecutive_good = 0
        else:
            self.consecutive_good = 0
        changed = abs(n_active - prev_n_active)
        if changed > 0:
            rate = changed / max(prev_n_active, n_active, 1)
            if rate > self.contact_change:
                nxt = min(nxt, current * self.shrink)
                self.consecutive_good = 0
        nxt = max(nxt, self.min_frac)
        nxt = min(nxt, self.max_frac)
        frac = min(load_frac + nxt, 1.0)
        if 1.0 - frac < self.min_frac * 0.5:
            frac = 1.0
        self.queue.appendleft(frac)

    def failure(self, load_frac: float, load_frac_prev: float, diverged: bool) -> bool:
        """True when the step may be retried with a smaller increment."""
        delta = load_frac - load_frac_prev
        if delta <= self.min_frac + 1e-15:
            return False
        self.consecutive_good = 0
        self.n_cutbacks += 1
        shrink = self.shrink * self.shrink if diverged else self.shrink
        self.queue.appendleft(load_frac)
        self.queue.appendleft(load_frac_prev + delta * shrink)
        return True


class ScheduledSteps(StepControl):
    """A fixed list of load fractions: no growth.  Used to put two runs on the same increments, e.g. the
    increments a reference run took.  A failed increment ends the run, or with ``cutbacks`` is retried
    from a shrunk fraction (as ``StepControl.failure``), after which the list continues."""

    def __init__(self, t_total: float, fractions, *, cutbacks: bool = False, min_frac: float = 0.0):
        super().__init__(t_total)
        fr = [float(f) for f in fractions]
        if not fr or any(b <= a for a, b in zip(fr, fr[1:])) or fr[0] <= 0.0 or abs(fr[-1] - 1.0) > 1e-12:
            raise ValueError("load schedule: increasing fractions in (0, 1], ending at 1")
        self.queue = deque(fr)
        self.cutbacks = cutbacks
        if min_frac > 0.0:
            self.min_frac = min_frac

    def success(self, load_frac, load_frac_prev, n_attempts, n_active, prev_n_active) -> None:
        self._last_prev = load_frac
        if self.queue and self.queue[0] <= load_frac + 1e-15:
            self.queue.popleft()

    def failure(self, load_frac, load_frac_prev, diverged) -> bool:
        delta = load_frac - load_frac_prev
        if not self.cutbacks or delta <= self.min_frac + 1e-15:
            return False
        self.n_cutbacks += 1
        shrink = self.shrink * self.shrink if diverged else self.shrink
        self.queue.appendleft(load_frac_prev + delta * shrink)  # the failed target stays next in line
        return True


# --------------------------------------------------------------------------- settings and results


@dataclass
class SolverSettings:
    """``ContactFrictionInputData``'s solver fields and the manager's step-control fields."""

    max_nr_attempts: int = 50
    tol_force: float = 1e-8
    tol_disp: float = 1e-8
    divergence_window: int = 5
    du_norm_cap: float = 0.0
    max_increments: int = 10000
    use_line_search: bool = True
    line_search_max_steps: int = 5
    dt_grow_factor: float = 1.5
    dt_shrink_factor: float = 0.5
    dt_grow_attempt_threshold: int = 5
    dt_shrink_attempt_threshold: int = 15
    dt_contact_change_threshold: float = 0.3
    dt_min_fraction: float = 0.0
    dt_max_fraction: float = 0.0
    # the energy test |du . R| / (its first value) < energy_tol (the reference's fixed 1e-10,
    # _newton_steps.py:229-235); 0 switches it off, so that only the force and displacement tests end
    # an increment (used where two runs are compared to a tighter tolerance than the energy test gives)
    energy_tol: float = 1e-10
    # the force test also passes when |R| <= residual_floor * |f_int|: the attainable residual of an engine
    # that assembles in float (about 1e-7 of the internal forces), which a relative test against a small
    # increment's first residual can ask below; 0 (the reference's test alone) for the FP64 engine
    residual_floor: float = 0.0
    # increments at exactly these load fractions (ScheduledSteps) instead of the adaptive control;
    # with schedule_cutbacks a failed one is retried from a shrunk fraction
    load_schedule: tuple = ()
    schedule_cutbacks: bool = False


@dataclass
class IncrementRecord:
    step: int
    load_frac: float
    dt: float
    converged: bool
    attempts: int
    n_active: int
    residuals: list
    convergence: str
    u: np.ndarray | None = None


@dataclass
class SolverResult:
    u: torch.Tensor
    converged: bool
    n_increments: int
    total_attempts: int
    n_cutbacks: int
    increments: list = field(default_factory=list)  # converged increments, in order
    attempts_log: list = field(default_factory=list)  # every increment tried, retries included

    @property
    def completed(self) -> bool:
        """Converged through the full load.  ``converged`` alone is also True when the run stopped at
        ``max_increments``, as the reference's is (``process.py:377-381,650-674``)."""
        return self.converged and bool(self.increments) and self.increments[-1].load_frac >= 1.0 - 1e-12


# --------------------------------------------------------------------------- linear solves


def dirichlet_solve_host(K: sp.spmatrix, R: np.ndarray, fixed: np.ndarray) -> np.ndarray | None:
    """``LinearSolveProcess`` (``_newton_steps.py:338-366``): zero the fixed rows and columns, put 1 on
    their diagonal, solve ``K du = -R`` with the fixed right-hand side zero; None when the solver raises."""
    K = K.tocsc()
    free = (~fixed).astype(float)
    D = sp.diags(free)
    Keff = (D @ K @ D + sp.diags(fixed.astype(float))).tocsc()
    Keff.eliminate_zeros()
    rhs = -R.copy()
    rhs[fixed] = 0.0
    try:
        return spla.spsolve(Keff, rhs)  # a singular matrix gives non-finite values, not an error, as there
    except Exception:  # noqa: BLE001 - the reference treats any solver error as a failed solve
        return None


class HostDirectSolve:
    """The reference's direct solve on the host, K copied back from the device every iteration."""

    def __call__(self, backend, R: torch.Tensor, fixed: np.ndarray, mass_diag: torch.Tensor | None):
        K = backend.K_csr()
        if mass_diag is not None:
            K = K + sp.diags(mass_diag.cpu().numpy())
        du = dirichlet_solve_host(K, R.cpu().numpy(), fixed)
        return None if du is None else torch.as_tensor(du, dtype=torch.float64, device=R.device)


# --------------------------------------------------------------------------- the GPU engine as a backend


class EngineBackend:
    """``AssemblyEngine`` in the solver's terms (FP64 or mixed engine).

    ``graph=True`` replays the assembly as a CUDA graph: the first assembly
    after a detection records it on static input buffers (the recording's
    warm-up launch is that attempt's assembly), the later attempts of the
    increment copy their inputs in and replay it.
    """

    def __init__(self, engine, graph: bool = False):
        self.eng = engine
        self.device = engine.device
        self.ndof = engine.mesh.ndof
        self.graph = graph
        self._fint = torch.zeros(self.ndof, dtype=torch.float64, device=self.device)
        self._static = None
        self.counts = {"detect": 0, "assemble": 0, "captures": 0, "replays": 0, "internal_force": 0}

    def detect(self, u: torch.Tensor) -> dict:
        self.counts["detect"] += 1
        return self.eng.detect(u)

    def assemble(self, u: torch.Tensor, u_ref: torch.Tensor, f_ext: torch.Tensor, fixed_u8: torch.Tensor):
        """(R, f_c): R = f_int + f_c - f_ext with fixed entries zero; f_c = -(f_n + f_f) on the free DOFs."""
        eng = self.eng
        self.counts["assemble"] += 1
        if not self.graph:
            R = eng.assemble(u, u_ref, f_ext, fixed_u8).clone()
        else:
            if self._static is None:
                self._static = tuple(torch.empty_like(t) for t in (u, u_ref, f_ext, fixed_u8))
            for dst, src in zip(self._static, (u, u_ref, f_ext, fixed_u8)):
                dst.copy_(src)
            if eng.graph is None:  # a detection dropped the graph: record it (its warm-up runs this assembly)
                eng.capture(*self._static)
                self.counts["captures"] += 1
            else:
                eng.replay()
                self.counts["replays"] += 1
            R = eng.R.clone()
        f_c = R + f_ext - eng.f_int
        return R, f_c

    def f_int_norm(self) -> float:
        """|f_int| of the last assembly."""
        return float(torch.linalg.vector_norm(self.eng.f_int))

    def internal_force(self, u: torch.Tensor) -> torch.Tensor:
        """f_int(u) alone, in the engine's precision (the line search's only assembly)."""
        eng = self.eng
        self.counts["internal_force"] += 1
        if eng.precision == L.XK_MIXED:
            import ctypes as C

            s = stream_handle(None)
            L.call("xk_nodes_prepare", C.byref(eng.mesh.c), ptr(u), ptr(u), ptr(eng.node32), s)
            L.call("xk_beam_assemble32", C.byref(eng.mesh.c), C.byref(eng.beam.section), ptr(eng.elem32),
                   C.byref(eng.beam.plan), ptr(eng.node32), ptr(self._fint), None, s)
        else:
            eng.beam.assemble(u, eng.precision, self._fint, None)
        return self._fint.clone()

    def n_active(self) -> int:
        """Pairs with p_n > 0 (``_newton_steps.py:199``)."""
        eng = self.eng
        n = eng.pairs.n
        if n == 0:
            return 0
        if eng._state_in32:
            return int((eng.pairs32.t["p_n"][:n] > 0).sum().item())
        return int((eng.pairs.t["p_n"][:n] > 0).sum().item())

    def K_csr(self) -> sp.csr_matrix:
        return self.eng.K_total_csr()


# --------------------------------------------------------------------------- the loop


class ContactFrictionSolver:
    """One run of the reference's contact solver: a ramp of the prescribed displacements and external
    loads over ``t_total`` (the physical time ``dt_physical``) in adaptive increments.

    ``dynamics`` is the time integrator (``GpuGeneralizedAlpha`` or any object with the reference's
    TimeIntegrationStrategy methods plus ``mass_coefficient(dt)`` and the lumped mass ``m``), or
    ``QuasiStatic()`` for a load step without inertia (the reference's loop is dynamic only,
    ``process.py:179-185``; without inertia its predictor, corrector and mass terms drop out);
    ``linear_solve(backend, R, fixed, mass_diag) -> du or None`` the linear solver.
    """

    def __init__(self, backend, dynamics, *, t_total: float, fixed_dofs=(), prescribed_dofs=(),
                 prescribed_values=(), prescribed_start=None, f_ext_total=None, f_ext_base=None,
                 settings: SolverSettings | None = None, linear_solve=None, record_u: bool = True,
                 verbose: bool = False):
        self.b = backend
        self.dyn = dynamics
        self.cfg = settings or SolverSettings()
        nd = backend.ndof
        dev = backend.device
        self.t_total = float(t_total)
        pd = np.asarray(prescribed_dofs, dtype=np.int64)
        fx = np.zeros(nd, dtype=bool)
        fx[np.asarray(fixed_dofs, dtype=np.int64)] = True
        fx[pd] = True  # prescribed DOFs are fixed DOFs with values (process.py:187-199)
        self.fixed = fx
        self.fixed_u8 = torch.as_tensor(fx.astype(np.uint8), device=dev)
        self.free = torch.as_tensor(~fx, device=dev)
        self.pd = torch.as_tensor(pd, device=dev)
        self.pv = torch.as_tensor(np.asarray(prescribed_values, dtype=np.float64), device=dev)
        # values at load fraction 0: zero as in the reference (u[dofs] = load_frac * values); a run that
        # continues from a driven state (the steps of an oscillation) ramps from where the last one ended
        self.p0 = torch.zeros_like(self.pv) if prescribed_start is None else torch.as_tensor(
            np.asarray(prescribed_start, dtype=np.float64), device=dev)
        z = torch.zeros(nd, dtype=torch.float64, device=dev)
        self.f_ext_total = z if f_ext_total is None else torch.as_tensor(f_ext_total, dtype=torch.float64,
                                                                          device=dev)
        self.f_ext_base = z if f_ext_base is None else torch.as_tensor(f_ext_base, dtype=torch.float64, device=dev)
        self.linear_solve = linear_solve or HostDirectSolve()
        self.record_u = record_u
        self.verbose = verbose

    # ------------------------------------------------------------ one increment's Newton iterations
    def _line_search(self, u, du, f_ext, f_c, res_norm) -> float:
        """``_ncp_line_search`` with ``diverge_factor = 3`` (``_utils.py:31-61``, ``_newton_steps.py:410-423``)."""
        alpha = 1.0
        for _ in range(self.cfg.line_search_max_steps):
            R = self.b.internal_force(u + alpha * du) + f_c - f_ext
            R = torch.where(self.free, R, torch.zeros((), dtype=R.dtype, device=R.device))
            if not bool(torch.isfinite(R).all()):
                alpha *= 0.5
                continue
            if float(torch.linalg.vector_norm(R)) < 3.0 * max(res_norm, 1e-30):
                return alpha
            alpha *= 0.5
        return alpha

    def _newton(self, u, u_ref, f_ext, dt_sub, f_ext_ref_norm, dynamic_ref):
        cfg, dyn, b = self.cfg, self.dyn, self.b
        zero = torch.zeros((), dtype=torch.float64, device=u.device)
        energy_ref = None
        incr_f_ref = 0.0
        prev_ratio = math.inf
        consecutive = 0
        n_active = 0
        hist = []
        attempts = 0
        f_c = torch.zeros_like(u)
        for att in range(cfg.max_nr_attempts):
            attempts += 1
            R, f_c = b.assemble(u, u_ref, f_ext, self.fixed_u8)
            if dt_sub > 1e-30 and dyn.is_dynamic:
                dyn.correct(u, None, dt_sub)
                R = dyn.effective_residual(R, dt_sub)
                R = torch.where(self.free, R, zero)
            # force test (ConvergenceCheckProcess, first call)
            eff_ref = incr_f_ref if incr_f_ref > 1e-30 else f_ext_ref_norm
            res = float(torch.linalg.vector_norm(R))
            f_ref = res if (dynamic_ref and att == 0 and res > 1e-30) else eff_ref
            n_active = b.n_active()
            if att == 0 and dynamic_ref:
                incr_f_ref = f_ref
            ratio = res / f_ref
            hist.append(ratio)
            if ratio < cfg.tol_force:
                return True, attempts, n_active, f_c, hist, "force", False
            if cfg.residual_floor > 0.0 and res <= cfg.residual_floor * b.f_int_norm():
                return True, attempts, n_active, f_c, hist, "floor", False
            # divergence (_newton_dynamic.py:262-283)
            if att > 0 and ratio > prev_ratio * 1.01:
                consecutive += 1
            else:
                consecutive = 0
            prev_ratio = ratio
            if (consecutive >= cfg.divergence_window and not ratio < 0.01) or (att >= 10 and ratio > 100.0):
                return False, attempts, n_active, f_c, hist, "diverged", True
            # tangent and solve
            mass = None
            if dt_sub > 1e-30 and dyn.is_dynamic:
                mass = dyn.mass_coefficient(dt_sub) * dyn.m
            du = self.linear_solve(b, R, self.fixed, mass)
            if du is None:
                return False, attempts, n_active, f_c, hist, "solve failed", False
            du = torch.where(self.free, du, zero)
            scale = 1.0
            if cfg.use_line_search:
                scale *= self._line_search(u, du, f_ext, f_c, res)
            if cfg.du_norm_cap > 0.0:
                dn = float(torch.linalg.vector_norm(scale * du))
                un = max(float(torch.linalg.vector_norm(u)), 1.0)
                if dn > cfg.du_norm_cap * un:
                    scale *= cfg.du_norm_cap * un / dn
            du = scale * du
            u += du
            # displacement and energy tests (ConvergenceCheckProcess, second call)
            eff_ref2 = incr_f_ref if incr_f_ref > 1e-30 else f_ext_ref_norm
            if res / eff_ref2 < cfg.tol_force:
                return True, attempts, n_active, f_c, hist, "force", False
            du_norm = float(torch.linalg.vector_norm(du))
            u_norm = float(torch.linalg.vector_norm(u))
            if u_norm > 1e-30 and du_norm / u_norm < cfg.tol_disp:
                return True, attempts, n_active, f_c, hist, "displacement", False
            energy = abs(float(torch.dot(du, R)))
            if energy_ref is None:
                energy_ref = energy if energy > 1e-30 else 1.0
            if cfg.energy_tol > 0.0 and energy_ref > 1e-30 and energy / energy_ref < cfg.energy_tol:
                return True, attempts, n_active, f_c, hist, "energy", False
        return False, attempts, n_active, f_c, hist, "max attempts", False

    # ------------------------------------------------------------ the step loop
    def run(self, u0=None) -> SolverResult:
        cfg, dyn, b = self.cfg, self.dyn, self.b
        dev = b.device
        nd = b.ndof
        u = torch.zeros(nd, dtype=torch.float64, device=dev) if u0 is None else \
            torch.as_tensor(u0, dtype=torch.float64, device=dev).clone()
        u_ref = u.clone()
        f_ext_ref_norm = float(torch.linalg.vector_norm(self.f_ext_total))
        dynamic_ref = f_ext_ref_norm < 1e-30
        if dynamic_ref:
            f_ext_ref_norm = 1.0
        t = self.t_total
        if cfg.load_schedule:
            ctl = ScheduledSteps(t, cfg.load_schedule, cutbacks=cfg.schedule_cutbacks,
                                 min_frac=cfg.dt_min_fraction)
        else:
            ctl = StepControl(t, t, cfg.dt_min_fraction * t if cfg.dt_min_fraction > 0 else t / 32.0,
                              cfg.dt_max_fraction * t if cfg.dt_max_fraction > 0 else t, cfg.dt_grow_factor,
                              cfg.dt_shrink_factor, cfg.dt_grow_attempt_threshold
                              if cfg.dt_grow_attempt_threshold > 0 else 5, cfg.dt_shrink_attempt_threshold,
                              cfg.dt_contact_change_threshold)
        ckpt = (u.clone(), u_ref.clone())
        dyn.checkpoint()
        load_prev = 0.0
        increment = 0
        total = 0
        prev_n_active = 0
        count = 0
        out = SolverResult(u, False, 0, 0, 0)
        while True:
            if cfg.max_increments > 0 and count >= cfg.max_increments:
                break
            more, lf, dt_sub = ctl.query(load_prev)
            if not more:
                break
            count += 1
            increment += 1
            f_ext = self.f_ext_base + lf * self.f_ext_total
            if dyn.is_dynamic:
                u = dyn.predict(u, dt_sub)
                if not isinstance(u, torch.Tensor):
                    u = torch.as_tensor(u, dtype=torch.float64, device=dev)
            if self.pd.numel():
                u[self.pd] = self.p0 + lf * (self.pv - self.p0)
            try:
                b.detect(u)
            except L.XkError:
                # a state the engine cannot take (e.g. a node in contact with more nodes than a pattern row
                # holds), reached from a bad prediction: the increment fails like a diverged one
                ok, att, n_active, f_c, hist, kind, diverged = False, 0, 0, None, [math.inf], "detection failed", True
            else:
                ok, att, n_active, f_c, hist, kind, diverged = self._newton(u, u_ref, f_ext, dt_sub,
                                                                            f_ext_ref_norm, dynamic_ref)
            total += att
            rec = IncrementRecord(increment, lf, dt_sub, ok, att, n_active, hist, kind)
            out.attempts_log.append(rec)
            if self.verbose:
                print(f"  incr {increment} frac {lf:.6f} attempts {att} active {n_active} {kind} "
                      f"res {hist[-1]:.3e}")
            if not ok:
                if ctl.failure(lf, load_prev, diverged):
                    u, u_ref = ckpt[0].clone(), ckpt[1].clone()
                    dyn.restore_checkpoint()
                    increment -= 1
                    continue
                out.u, out.converged = u, False
                out.n_increments, out.total_attempts, out.n_cutbacks = increment, total, ctl.n_cutbacks
                return out
            if dt_sub > 1e-30 and dyn.is_dynamic:
                dyn.correct(u, None, dt_sub)
            ctl.success(lf, load_prev, att, n_active, prev_n_active)
            prev_n_active = n_active
            load_prev = lf
            u_ref = u.clone()
            ckpt = (u.clone(), u_ref.clone())
            dyn.checkpoint()
            if self.record_u:
                rec.u = u.cpu().numpy()
            out.increments.append(rec)
        out.u, out.converged = u, True
        out.n_increments, out.total_attempts, out.n_cutbacks = increment, total, ctl.n_cutbacks
        return out
