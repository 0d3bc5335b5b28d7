"""The device block-tridiagonal solve of the Newton system against the reference's host direct solve.

``BlockTridiagonalSolver`` (GMRES in FP64 on the engine's SpMV, preconditioned by the float32 block LU
of the axially ordered system) must give the ``du`` of ``LinearSolveProcess``'s sparse direct solve
(``xkep_cae/contact/solver/_newton_steps.py:338-366``) on a strand system with active contacts, with
and without the time integrator's mass term, and must keep doing so when its factors are kept from an
earlier system (a later Newton iteration at another state): the relative residual of the reduced system
within 1e-9, and ``du`` within 1e-6 of the host solution (measured: 2e-8; the systems' conditioning
times the residuals of the two solves).
"""

from __future__ import annotations

import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from xkgpu import runs, workloads as W  # noqa: E402
from xkgpu.blocktri import BlockTridiagonalSolver  # noqa: E402
from xkgpu.solver import EngineBackend, HostDirectSolve  # noqa: E402


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_block_solve_matches_host_direct_solve(precision):
    w = W.strand_workload("strand19", 19, 2.0, 40.0, 1, 24, gap_frac=-0.005, seed=3)
    eng = runs.strand_engine(w, precision)
    b = EngineBackend(eng)
    st = w.strand
    fixed = np.zeros(st.ndof, dtype=bool)
    fixed[runs.bending_boundary(st, 1e-3)[0]] = True
    fixed_u8 = torch.as_tensor(fixed.astype(np.uint8), device="cuda")
    zero = torch.zeros(st.ndof, dtype=torch.float64, device="cuda")
    mass = runs.lumped_mass(eng) * 3.6e8  # c0 M at dt = 1e-4 s, rho_inf = 0.9
    lin = BlockTridiagonalSolver(eng, refactor_iters=1000)
    host = HostDirectSolve()
    rng = np.random.default_rng(5)
    u = torch.as_tensor(w.u, device="cuda")
    b.detect(u)
    assert b.n_active() > 0 or eng.pairs.n > 0
    for k, m in enumerate([None, mass, mass, None]):
        if k:  # a later iterate: another K, the factors kept from the first solve
            u = u + torch.as_tensor(rng.normal(0.0, 1e-4, st.ndof), device="cuda") * torch.as_tensor(
                ~fixed, device="cuda")
        R, _ = b.assemble(u, u, zero, fixed_u8)
        du = lin(b, R, fixed, m)
        want = host(b, R, fixed, m)
        # the Krylov residual of the Dirichlet-reduced system, with the host's K
        K = b.K_csr()
        if m is not None:
            K = K + sp.diags(m.cpu().numpy())
        x = du.cpu().numpy()
        rhs = np.where(fixed, 0.0, -R.cpu().numpy())
        res = np.where(fixed, x, K @ np.where(fixed, 0.0, x)) - rhs
        assert np.linalg.norm(res) <= 1e-9 * np.linalg.norm(rhs), (k, np.linalg.norm(res) / np.linalg.norm(rhs))
        # the two solutions differ by the systems' conditioning times their residuals
        err = float(torch.max(torch.abs(du - want)) / torch.max(torch.abs(want)))
        assert err <= 1e-6, (k, err)
    assert lin.stats["factorizations"] + lin.stats["stale_refactor"] >= 1
    assert lin.stats["not_converged"] == 0
