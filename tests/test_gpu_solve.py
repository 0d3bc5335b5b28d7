"""The Newton step's linear solve on the device against scipy's direct solve.

``LinearSolveProcess`` (xkep_cae/contact/solver/_newton_steps.py:338-366)
solves ``K du = -R`` with the Dirichlet DOFs' rows and columns set to the
identity by a sparse direct factorisation.  The device solve (block-Jacobi
BiCGStab on the engine's K_beam and K_c) must give the same increment to the
solver tolerance, the same bits on every run, and the same Newton path.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

import scipy.sparse.linalg as spla  # noqa: E402

from test_gpu_newton import _strand7  # noqa: E402
from xkgpu.dynamics import GpuGeneralizedAlpha  # noqa: E402
from xkgpu.newton import _dirichlet, solve_increment  # noqa: E402
from xkgpu.solve import DeviceLinearSolver  # noqa: E402


def _assembled(prec):
    w, eng, fixed = _strand7(prec)
    u = torch.zeros(eng.mesh.ndof, dtype=torch.float64, device="cuda")
    eng.detect(u)
    R = eng.assemble(u, u, None, torch.as_tensor(fixed.astype(np.uint8), device="cuda"))
    torch.cuda.synchronize()
    assert eng.pattern.nnzb > 0  # the contact tangent takes part
    return eng, fixed, R


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_spmv_matches_host_matrix(prec):
    eng, fixed, _ = _assembled(prec)
    ds = DeviceLinearSolver(eng)
    ds.set_fixed(fixed)
    A = _dirichlet(eng.K_total_csr(), fixed)
    x = np.random.default_rng(3).normal(size=eng.mesh.ndof)
    y = ds.matvec(torch.as_tensor(x, device="cuda")).cpu().numpy()
    ref = A @ x
    assert rel_err(y, ref) < 1e-13


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_bicgstab_matches_direct_solve(prec):
    eng, fixed, R = _assembled(prec)
    ds = DeviceLinearSolver(eng, rtol=1e-12, max_iter=5000)
    ds.set_fixed(fixed)
    rhs = -R.double().cpu().numpy()
    rhs[fixed] = 0.0
    x_ref = spla.spsolve(_dirichlet(eng.K_total_csr(), fixed), rhs)
    b = torch.as_tensor(rhs, device="cuda")
    x = ds.solve(b)
    print(prec, "iterations", ds.iterations, "relative residual", ds.rel_res)
    assert ds.rel_res <= 1e-12
    assert rel_err(x.cpu().numpy(), x_ref) < 1e-7
    x2 = ds.solve(b)
    assert torch.equal(x, x2)  # fixed-order reductions: the same bits on every run


@pytest.mark.parametrize("graph", [False, True])
def test_quasi_static_newton_device_solve_matches_host_solve(graph):
    """With ``graph=True`` the whole iteration stays on the device: the replayed assembly graph, the
    device solve and the update; the host reads only the residual norm and the solver's checks."""
    out = {}
    for solver in (None, "device"):
        w, eng, fixed = _strand7("fp64")
        u0 = torch.zeros(eng.mesh.ndof, dtype=torch.float64, device="cuda")
        out[solver] = solve_increment(eng, u0, u0, fixed=fixed, tol=1e-9, max_iter=25, solver=solver,
                                      graph=graph and solver == "device")
        print(solver, out[solver].iterations, ["%.2e" % r for r in out[solver].residuals])
    assert out[None].converged and out["device"].converged
    assert abs(out["device"].iterations - out[None].iterations) <= 1
    assert rel_err(out["device"].u.cpu().numpy(), out[None].u.cpu().numpy()) < 1e-7


def test_dynamic_newton_device_solve_matches_host_solve():
    us = {}
    for solver in (None, "device"):
        w, eng, fixed = _strand7("fp64")
        nd = eng.mesh.ndof
        m = torch.zeros(nd, dtype=torch.float64, device="cuda")
        eng.beam.lumped_mass(7.85e-9, m)
        ga = GpuGeneralizedAlpha(m, rho_inf=0.9)
        v0 = np.zeros((nd // 6, 6))
        v0[:, 0] = 50.0
        v0 = v0.ravel()
        v0[fixed] = 0.0
        ga.set_initial_state(velocity=v0)
        u = torch.zeros(nd, dtype=torch.float64, device="cuda")
        for _ in range(2):
            res = solve_increment(eng, u, u, fixed=fixed, dynamics=ga, dt=1e-4, tol=1e-9, max_iter=20,
                                  solver=solver)
            assert res.converged
            u = res.u
        us[solver] = u.cpu().numpy()
    assert rel_err(us["device"], us[None]) < 1e-7


def test_unconverged_solve_raises():
    """At the workload state (initial penetration, k_pen = 1e3 EA/L, mu = 0.1) the tangent is indefinite:
    a short solve must raise instead of returning an unconverged increment."""
    from xkgpu import workloads as W
    from xkgpu.engine import AssemblyEngine
    from xkgpu.solve import LinearSolveError

    w = W.config_workload("strand7", seed=0)
    st = w.strand
    eng = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision="fp64", **w.engine_kwargs())
    u = torch.as_tensor(w.u, device="cuda")
    eng.detect(u)
    R = eng.assemble(u, u)
    ds = DeviceLinearSolver(eng, rtol=1e-12, max_iter=50)
    with pytest.raises(LinearSolveError):
        ds.solve(-R.double())
    assert 0 < ds.iterations <= 50 and not ds.rel_res <= 1e-12
