"""Newton iterations of one increment over the device assembly.

A compact driver in the shape of ``NewtonDynamicProcess``
(``xkep_cae/contact/solver/_newton_dynamic.py:115-398``): detection and the
active-set update at the start of the increment, then per iteration the GPU
assembly (``AssemblyEngine.assemble``: R and K_T), the time integrator's
effective residual / stiffness, the convergence check and a linear solve with
the Dirichlet DOFs eliminated (rows and columns replaced by the identity, as
``LinearSolveProcess``, ``_newton_steps.py:338-366``).  The linear solve runs on
the host (scipy by default, or any ``solver(K, rhs)``), or with
``solver="device"`` on the GPU (``DeviceLinearSolver``: BiCGStab on the
engine's block matrices), so that no matrix leaves the device.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla
import torch

from .dynamics import QuasiStatic
from .solve import DeviceLinearSolver


@dataclass
class NewtonResult:
    u: torch.Tensor
    converged: bool
    iterations: int
    residuals: list = field(default_factory=list)


def _dirichlet(K: sp.csr_matrix, fixed: np.ndarray) -> sp.csr_matrix:
    if not fixed.any():
        return K
    free = sp.diags((~fixed).astype(float))
    return (free @ K @ free + sp.diags(fixed.astype(float))).tocsc()


def solve_increment(engine, u_start: torch.Tensor, u_ref: torch.Tensor, *, f_ext: torch.Tensor | None = None,
                    fixed: np.ndarray | None = None, dynamics=None, dt: float = 0.0, tol: float = 1e-8,
                    max_iter: int = 30, f_ref: float | None = None, solver=None, detect: bool = True,
                    graph: bool = False) -> NewtonResult:
    """Run Newton iterations from ``u_start`` (Dirichlet values already set in it).

    Convergence: ``||R|| <= tol * f_ref`` with ``f_ref`` the first residual norm
    unless given.  ``fixed``: boolean per DOF (host).  ``graph``: record the
    assembly once as a CUDA graph on static buffers and replay it every
    iteration.  ``solver``: ``None`` (scipy's direct solve), ``"device"`` (a
    ``DeviceLinearSolver``), a ``DeviceLinearSolver`` instance, or any host
    ``solver(K, rhs)``.
    """
    dyn = dynamics if dynamics is not None else QuasiStatic()
    dsolve = None
    if isinstance(solver, DeviceLinearSolver):
        dsolve = solver
    elif isinstance(solver, str):
        if solver != "device":
            raise ValueError(f"unknown solver {solver!r}")
        dsolve = DeviceLinearSolver(engine)
    solve = solver if callable(solver) and dsolve is None else (lambda K, b: spla.spsolve(K, b))
    nd = engine.mesh.ndof
    fx = np.zeros(nd, dtype=bool) if fixed is None else np.asarray(fixed, dtype=bool)
    fx_dev = torch.as_tensor(fx.astype(np.uint8), device=engine.device)
    free_dev = torch.as_tensor(~fx, device=engine.device)
    if dsolve is not None:
        dsolve.set_fixed(fx)
    if detect:
        engine.detect(u_start)
    u = dyn.predict(u_start, dt) if dyn.is_dynamic else u_start.clone()
    u = torch.where(free_dev, u, u_start)  # the prescribed values stay
    if graph:
        u_in, ur_in = u.clone(), u_ref.clone()
        engine.capture(u_in, ur_in, f_ext, fx_dev)
    history = []
    for it in range(max_iter + 1):
        if dyn.is_dynamic:
            dyn.correct(u, None, dt)
        if graph:
            u_in.copy_(u)
            engine.replay()
            R = engine.R
        else:
            R = engine.assemble(u, u_ref, f_ext, fx_dev)
        if dyn.is_dynamic:
            R = dyn.effective_residual(R, dt)
            R = torch.where(free_dev, R, torch.zeros_like(R))
        norm = float(torch.linalg.vector_norm(R).item())
        history.append(norm)
        ref = f_ref if f_ref is not None else max(history[0], 1e-300)
        if norm <= tol * ref:
            return NewtonResult(u, True, it, history)
        if it == max_iter:
            break
        if dsolve is not None:
            if dyn.is_dynamic:
                dyn.add_mass_to(engine.K_beam, engine.beam.diag_index(), dt, engine.precision)
            rhs = torch.where(free_dev, -R.to(torch.float64), torch.zeros((), dtype=torch.float64,
                                                                            device=engine.device))
            du = dsolve.solve(rhs)
            u = u + torch.where(free_dev, du, torch.zeros_like(du))
            continue
        K = engine.K_total_csr()
        if dyn.is_dynamic:
            K = dyn.effective_stiffness(K, dt)
        du = solve(_dirichlet(K.tocsr(), fx), -R.cpu().numpy())
        du[fx] = 0.0
        u = u + torch.as_tensor(du, device=engine.device)
    return NewtonResult(u, False, max_iter, history)
