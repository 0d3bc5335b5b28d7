"""Time integration and Newton iterations over the device assembly.

The Generalized-alpha kernels against the reference's recorded outputs, and
full Newton solves (quasi-static and dynamic) in FP64 and in mixed precision:
the converged displacements of the two agree to 1e-6 relative.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from xkgpu import workloads as W  # noqa: E402
from xkgpu.dynamics import GpuGeneralizedAlpha  # noqa: E402
from xkgpu.engine import AssemblyEngine  # noqa: E402
from xkgpu.newton import solve_increment  # noqa: E402


def test_genalpha_kernels_match_reference():
    z = golden("genalpha")
    m = z["m"]
    rng = np.random.default_rng(4)
    rng.uniform(1e-9, 1e-6, m.size)
    for rho, tag in ((0.9, "r09"), (0.5, "r05")):
        ga = GpuGeneralizedAlpha(m, rho_inf=rho)
        ga.set_initial_state(velocity=rng.normal(size=m.size), acceleration=rng.normal(size=m.size) * 1e3)
        rng.normal(size=m.size)
        for step in range(3):
            p = f"{tag}_s{step}_"
            dt = float(z[p + "dt"])
            assert rel_err(ga.predict(z[p + "u"], dt), z[p + "u_pred"]) < 1e-15
            ga.correct(z[p + "u1"], None, dt)
            assert rel_err(ga.acc.cpu().numpy(), z[p + "acc"]) < 1e-12
            assert rel_err(ga.vel.cpu().numpy(), z[p + "vel"]) < 1e-12
            assert rel_err(ga.effective_residual(z[p + "R"], dt), z[p + "R_eff"]) < 1e-14
            K = np.zeros(m.size)
            idx = torch.arange(m.size, device="cuda", dtype=torch.int64)
            Kd = torch.zeros(m.size, dtype=torch.float64, device="cuda")
            ga.add_mass_to(Kd, idx, dt, 0)
            assert rel_err(Kd.cpu().numpy(), z[p + "K_eff_diag"] - K) < 1e-12
            rng.normal(size=m.size)
            rng.normal(size=m.size)


def _strand7(precision):
    """The 7-wire strand with its initial penetration (gap -0.005 d), frictionless, k_pen = 1e4 N/mm.

    A well-posed equilibrium for plain Newton: the wires separate against their
    bending stiffness (with friction the return mapping rewrites z_t from the
    increment's total slip at every iteration, and Newton without the
    reference's line search and step control does not settle)."""
    w = W.config_workload("strand7", seed=0)
    st = w.strand
    kw = w.engine_kwargs()
    kw.update(k_pen=1e4, mu=0.0)
    eng = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision=precision, **kw)
    nw = len(st.wires)
    npw = st.n_elems_per_wire + 1
    fixed = np.zeros((st.n_nodes, 6), dtype=bool)
    for wi in range(nw):
        fixed[wi * npw] = True
        fixed[wi * npw + npw - 1] = True
    return w, eng, fixed.ravel()


@pytest.mark.parametrize("graph", [False, True])
def test_quasi_static_newton_mixed_matches_fp64(graph):
    """Initial penetration of the 7-wire strand (gap -0.005 d) relaxed to equilibrium with clamped ends."""
    out = {}
    for prec in ("fp64", "mixed"):
        w, eng, fixed = _strand7(prec)
        u0 = torch.zeros(eng.mesh.ndof, dtype=torch.float64, device="cuda")
        # mixed precision reaches a residual floor near 4e-7 of the first residual
        res = solve_increment(eng, u0, u0, fixed=fixed, tol=1e-9 if prec == "fp64" else 1e-6, max_iter=25,
                              graph=graph)
        out[prec] = res
        print(prec, "converged", res.converged, "iterations", res.iterations,
              "residuals", ["%.2e" % r for r in res.residuals])
    assert out["fp64"].converged and out["mixed"].converged
    u64, umx = out["fp64"].u.cpu().numpy(), out["mixed"].u.cpu().numpy()
    assert np.max(np.abs(u64)) > 0
    d = rel_err(umx, u64)
    print("converged displacement, mixed vs fp64 (max-norm relative):", d)
    assert d < 1e-6


def test_dynamic_newton_mixed_matches_fp64():
    """Three Generalized-alpha steps (rho_inf 0.9, dt 1e-4 s) from a transverse initial velocity."""
    us = {}
    for prec in ("fp64", "mixed"):
        w, eng, fixed = _strand7(prec)
        nd = eng.mesh.ndof
        m = torch.zeros(nd, dtype=torch.float64, device="cuda")
        eng.beam.lumped_mass(7.85e-9, m)
        ga = GpuGeneralizedAlpha(m, rho_inf=0.9)
        v0 = np.zeros((nd // 6, 6))
        v0[:, 0] = 50.0  # mm/s
        v0 = v0.ravel()
        v0[fixed] = 0.0
        ga.set_initial_state(velocity=v0)
        u = torch.zeros(nd, dtype=torch.float64, device="cuda")
        for step in range(3):
            ga.checkpoint()
            res = solve_increment(eng, u, u, fixed=fixed, dynamics=ga, dt=1e-4,
                                  tol=1e-9 if prec == "fp64" else 1e-6, max_iter=20)
            assert res.converged
            u = res.u
        us[prec] = u.cpu().numpy()
    assert np.max(np.abs(us["fp64"])) > 0
    d = rel_err(us["mixed"], us["fp64"])
    print("dynamic displacement after 3 steps, mixed vs fp64:", d)
    assert d < 1e-6
