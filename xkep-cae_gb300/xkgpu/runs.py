"""Strand runs of the benchmark configurations over ``ContactFrictionSolver``.

* ``end_arc_values`` / ``bending_boundary``: a strand clamped at z = 0 whose
  z = L wire ends are driven to the section of a circular arc of curvature
  kappa about the x axis (end rotation kappa L, the section rotated rigidly
  about the arc's end point).
* ``compression_boundary``: the quasi-static load step of the 37-wire strand:
  every node of the outer layer moved radially inward (its x and y
  prescribed), the inner wires clamped at both ends, the outer wires' axial
  and rotational DOFs clamped at z = 0 only.
* ``run_bend_oscillation``: the 91-wire run: a quasi-static bend to the
  curvature, then the driven ends are released and the strand oscillates
  freely under Generalized-alpha, each time step one solver run that continues
  from the last (integrator state and pair state carried over).

The reference has no strand runner (its ``run_bending_oscillation`` is
imported but never defined, ``numerical_tests/wire_bending_benchmark.py:191-212``),
so these drivers are this package's own, over the restated solver loop.
"""

from __future__ import annotations

import dataclasses
import math
import time

import numpy as np
import torch

from .blocktri import BlockTridiagonalSolver
from .dynamics import GpuGeneralizedAlpha, QuasiStatic
from .engine import AssemblyEngine
from .solver import ContactFrictionSolver, EngineBackend, SolverSettings
from .strand import Strand

RHO_STEEL = 7.85e-9  # t/mm^3


def _wire_ends(strand: Strand):
    npw = strand.n_elems_per_wire + 1
    for w in strand.wires:
        n0 = w.wire_id * npw
        yield w, n0, n0 + npw - 1


def end_arc_values(strand: Strand, kappa: float) -> tuple[np.ndarray, np.ndarray]:
    """Prescribed DOFs and values that put every wire's z = L end on the section of an arc of curvature
    kappa (bending about x, the strand axis along z from the origin)."""
    L = strand.length
    phi = kappa * L
    pd, pv = [], []
    for _, _, ne in _wire_ends(strand):
        y = strand.coords[ne, 1]
        if abs(kappa) > 0.0:
            dyc, dzc = -(1.0 - math.cos(phi)) / kappa, math.sin(phi) / kappa - L
        else:
            dyc, dzc = 0.0, 0.0
        vals = [0.0, dyc + y * (math.cos(phi) - 1.0), dzc + y * math.sin(phi), phi, 0.0, 0.0]
        pd += [6 * ne + k for k in range(6)]
        pv += vals
    return np.asarray(pd, dtype=np.int64), np.asarray(pv, dtype=np.float64)


def arc_displacement(strand: Strand, kappa: float) -> np.ndarray:
    """Displacement that puts the whole strand on a circular arc of curvature kappa about x: every
    cross-section at height z turned rigidly by kappa z about x and carried to the arc (the bent
    state of the bending runs, rotations up to kappa L with little deformation)."""
    X = strand.coords
    phi = kappa * X[:, 2]
    if abs(kappa) > 0.0:
        cy, cz = -(1.0 - np.cos(phi)) / kappa, np.sin(phi) / kappa
    else:
        cy, cz = np.zeros_like(phi), X[:, 2].copy()
    u = np.zeros(strand.ndof)
    uu = u.reshape(-1, 6)
    uu[:, 1] = cy + X[:, 1] * np.cos(phi) - X[:, 1]
    uu[:, 2] = cz + X[:, 1] * np.sin(phi) - X[:, 2]
    uu[:, 3] = phi
    return u


def bending_boundary(strand: Strand, kappa: float):
    """(fixed DOFs, prescribed DOFs, values): z = 0 ends clamped, z = L ends on the arc section."""
    fixed = [6 * n0 + k for _, n0, _ in _wire_ends(strand) for k in range(6)]
    pd, pv = end_arc_values(strand, kappa)
    return np.asarray(fixed, dtype=np.int64), pd, pv


def compression_boundary(strand: Strand, layer: int, amount: float):
    """(fixed, prescribed, values) of the radial compression load step of ``layer`` by ``amount``."""
    npw = strand.n_elems_per_wire + 1
    fixed, pd, pv = [], [], []
    for w, n0, ne in _wire_ends(strand):
        if w.layer != layer:
            fixed += [6 * n0 + k for k in range(6)] + [6 * ne + k for k in range(6)]
            continue
        fixed += [6 * n0 + k for k in (2, 3, 4, 5)]
        for i in range(n0, n0 + npw):
            x, y = strand.coords[i, 0], strand.coords[i, 1]
            r = math.hypot(x, y)
            pd += [6 * i, 6 * i + 1]
            pv += [-amount * x / r, -amount * y / r]
    return np.asarray(fixed, dtype=np.int64), np.asarray(pd, dtype=np.int64), np.asarray(pv, dtype=np.float64)


def strand_engine(w, precision: str, **kw) -> AssemblyEngine:
    st = w.strand
    return AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision=precision, **w.engine_kwargs(), **kw)


def lumped_mass(engine: AssemblyEngine, rho: float = RHO_STEEL) -> torch.Tensor:
    m = torch.zeros(engine.mesh.ndof, dtype=torch.float64, device=engine.device)
    engine.beam.lumped_mass(rho, m)
    return m


def run_load_step(w, precision: str, *, layer: int, amount: float, settings: SolverSettings | None = None,
                  graph: bool = True, u0=None, verbose: bool = False):
    """The quasi-static radial-compression load step (no inertia); returns (result, backend, seconds)."""
    eng = strand_engine(w, precision)
    fixed, pd, pv = compression_boundary(w.strand, layer, amount)
    b = EngineBackend(eng, graph=graph)
    lin = BlockTridiagonalSolver(eng)
    b.lin_stats = lin.stats
    sol = ContactFrictionSolver(b, QuasiStatic(), t_total=1.0, fixed_dofs=fixed, prescribed_dofs=pd,
                                prescribed_values=pv, settings=settings or SolverSettings(dt_max_fraction=0.1),
                                linear_solve=lin, verbose=verbose)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = sol.run(u0)
    torch.cuda.synchronize()
    return res, b, time.perf_counter() - t0


def _closed(fracs) -> tuple:
    """A followed schedule that ends short of 1 (the run it came from failed there) gets the full load as
    its last increment, which then fails as well instead of being skipped."""
    f = tuple(float(x) for x in fracs)
    return f if f and abs(f[-1] - 1.0) <= 1e-12 else f + (1.0,)


def run_bend_oscillation(w, precision: str, *, kappa: float, dt: float = 1e-4, n_steps: int = 20,
                         rho_inf: float = 0.9, rho: float = RHO_STEEL, bend_time: float | None = None,
                         bend_settings: SolverSettings | None = None, step_settings: SolverSettings | None = None,
                         follow: list | None = None, graph: bool = True, verbose: bool = False):
    """Bend to the arc of curvature ``kappa`` (z = L wire ends driven to the arc's end section, z = 0 ends
    clamped), then release the z = L ends and take ``n_steps`` Generalized-alpha steps of ``dt``: the strand
    springs back in free oscillation, its contacts sliding and separating.  The bend is quasi-static
    (``bend_time`` None) or a Generalized-alpha run of ``bend_time`` from rest whose end state (velocities
    included) the oscillation continues.  Each oscillation step is one solver run continuing from the
    last (integrator state and pair state carried over).  ``follow``: the ``schedule`` of an earlier run
    (the load fractions of the bend's and of every step's increments), taken instead of the adaptive step
    control (an increment that fails is cut back and the list then continues), so that two runs (FP64
    and mixed) are compared at the same load fractions.

    Returns a dict: the displacements at the end of the bend and of every step (and of every bend
    increment), the schedule, the Newton attempt counts, the time spent in the solver runs and in the
    linear solves, and the assembly counts.
    """
    eng = strand_engine(w, precision)
    st = w.strand
    fixed, pd, pv = bending_boundary(st, kappa)
    b = EngineBackend(eng, graph=graph)
    lin = BlockTridiagonalSolver(eng)
    timing = {"solve_s": 0.0, "solves": 0}

    def timed_solve(backend, R, fx, mass):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        du = lin(backend, R, fx, mass)
        torch.cuda.synchronize()
        timing["solve_s"] += time.perf_counter() - t0
        timing["solves"] += 1
        return du

    out = {"u": [], "attempts": [], "step_s": [], "increments": []}

    def finish(converged, t0):
        torch.cuda.synchronize()
        out["converged"] = converged
        out["wall_s"] = time.perf_counter() - t0
        out.update(timing)
        out["counts"] = dict(b.counts)
        out["lin"] = dict(lin.stats)
        return out

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ga = GpuGeneralizedAlpha(lumped_mass(eng, rho), rho_inf=rho_inf, device=eng.device)
    if bend_time is None:
        dyn, t_bend = QuasiStatic(), 1.0
        bs = bend_settings or SolverSettings(dt_max_fraction=0.1)
    else:
        dyn, t_bend = ga, float(bend_time)
        bs = bend_settings or SolverSettings(dt_max_fraction=min(1.0, dt / t_bend))
    if follow is not None:
        bs = dataclasses.replace(bs, load_schedule=_closed(follow[0]), schedule_cutbacks=True)
    sol = ContactFrictionSolver(b, dyn, t_total=t_bend, fixed_dofs=fixed, prescribed_dofs=pd,
                                prescribed_values=pv, settings=bs, linear_solve=timed_solve, record_u=True,
                                verbose=verbose)
    res = sol.run()
    out["bend"] = {"increments": res.n_increments, "attempts": res.total_attempts, "cutbacks": res.n_cutbacks,
                   "converged": res.completed, "load_frac": [r.load_frac for r in res.increments]}
    out["bend_u"] = [r.u for r in res.increments]
    out["schedule"] = [[r.load_frac for r in res.increments]]
    out["u"].append(res.u.cpu().numpy())
    out["attempts"].append([r.attempts for r in res.increments])
    if not res.completed:
        return finish(False, t0)
    torch.cuda.synchronize()
    out["bend_s"] = time.perf_counter() - t0
    u = res.u
    clamped = fixed  # the z = L ends are released
    for k in range(n_steps):
        ts = time.perf_counter()
        ss = step_settings or SolverSettings()
        if follow is not None:
            if k + 1 >= len(follow):
                break
            ss = dataclasses.replace(ss, load_schedule=_closed(follow[k + 1]), schedule_cutbacks=True)
        sol = ContactFrictionSolver(b, ga, t_total=dt, fixed_dofs=clamped, settings=ss,
                                    linear_solve=timed_solve, record_u=False, verbose=verbose)
        r = sol.run(u)
        out["attempts"].append([x.attempts for x in r.increments])
        out["increments"].append(r.n_increments)
        out["schedule"].append([x.load_frac for x in r.increments])
        if not r.completed:
            return finish(False, t0)
        u = r.u
        out["u"].append(u.cpu().numpy())
        torch.cuda.synchronize()
        out["step_s"].append(time.perf_counter() - ts)
    return finish(True, t0)


def oscillation_states(w, kappa0: float, n_steps: int, *, jitter: float = 3e-4, seed: int = 7):
    """Displacements of a prescribed bending oscillation: at step k the strand lies on the arc of
    curvature kappa0 cos(2 pi k / n_steps) (rigid cross-sections), plus the workload's seeded noise and a
    fresh translation jitter of ``jitter`` d per step, which moves pairs across the contact threshold."""
    st = w.strand
    rng = np.random.default_rng(seed)
    mask = np.tile([1.0, 1.0, 1.0, 0.0, 0.0, 0.0], st.n_nodes)
    for k in range(n_steps):
        kap = kappa0 * math.cos(2.0 * math.pi * k / n_steps)
        yield w.u + arc_displacement(st, kap) + rng.normal(0.0, jitter * w.meta["d"], st.ndof) * mask


def run_detection_oscillation(w, kappa0: float, *, n_steps: int = 30, iterations: int = 2, pruner=None,
                              verify_every: int = 10, precision: str = "mixed", seed: int = 7):
    """Detection and Newton-iteration assemblies along a prescribed bending oscillation.

    Every step: one detection (pruned by ``pruner`` when given, the exact path verifying it every
    ``verify_every`` detections), then ``iterations`` graph-replayed assemblies at states jittered around
    the step's displacement.  Returns per-step times (ms) and the engine's pruning statistics.
    """
    eng = strand_engine(w, precision)
    if pruner is not None:
        eng.set_pruner(pruner, verify_every=verify_every)
    eng.trace_phases = True
    dev = eng.device
    nd = eng.mesh.ndof
    u_in = torch.zeros(nd, dtype=torch.float64, device=dev)
    ur_in = torch.zeros(nd, dtype=torch.float64, device=dev)
    rng = np.random.default_rng(seed + 1)
    mask = np.tile([1.0, 1.0, 1.0, 0.0, 0.0, 0.0], w.strand.n_nodes)
    out = {"detect_ms": [], "assemble_ms": [], "pairs": [], "members": [], "kept_candidates": [], "candidates": [],
           "phases_ms": []}
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    for k, uk in enumerate(oscillation_states(w, kappa0, n_steps, seed=seed)):
        ud = torch.as_tensor(uk, device=dev)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        stats = eng.detect(ud)
        torch.cuda.synchronize()
        out["detect_ms"].append(1e3 * (time.perf_counter() - t0))
        out["phases_ms"].append(eng.phase_ms())
        for key in ("pairs", "members", "kept_candidates", "candidates"):
            out[key].append(stats[key])
        ur_in.copy_(ud)
        u_in.copy_(ud)
        eng.capture(u_in, ur_in)
        tot = 0.0
        for _ in range(iterations):
            u_in.copy_(torch.as_tensor(uk + rng.normal(0.0, 1e-4 * w.meta["d"], nd) * mask, device=dev))
            ev[0].record()
            eng.replay()
            ev[1].record()
            ev[1].synchronize()
            tot += ev[0].elapsed_time(ev[1])
        out["assemble_ms"].append(tot / iterations)
    out["prune_stats"] = dict(eng.prune_stats)
    out["R_last"] = eng.R.clone()
    return out
