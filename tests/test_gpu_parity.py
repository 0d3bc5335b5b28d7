"""GPU path against the golden vectors and the oracle (through the C ABI).

Tolerances: FP64 mode 1e-10 relative (max-norm), mixed mode 1e-5 relative;
candidate sets, active sets and narrowphase results of the exact kernels are
compared bit for bit.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import golden, golden_csr, rel_err, sparse_rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # collected on CPU-only hosts, skipped there
    pytest.skip("no CUDA device", allow_module_level=True)

from oracle import beam as ob  # noqa: E402
from oracle import contact as oc  # noqa: E402
from xkgpu import _lib as L  # noqa: E402
from xkgpu.device import DeviceBeam, DeviceMesh, DevicePairTable  # noqa: E402
from xkgpu.engine import AssemblyEngine  # noqa: E402

SECTION_KEYS = ["E", "G", "A", "Iy", "Iz", "J", "kappa_y", "kappa_z"]
TOL64, TOLMIX = 1e-10, 1e-5


def _sec(z, scf=None):
    d = {k: float(z[k]) for k in SECTION_KEYS}
    d["scf"] = scf
    return d


def _dev(x, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=dtype, device="cuda")


def _beam_eval(coords, conn, u, sec, precision, v_ref=None):
    mesh = DeviceMesh(coords, conn, 0.0)
    beam = DeviceBeam(mesh, sec, v_ref=v_ref)
    f = torch.zeros(mesh.ndof, dtype=torch.float64, device="cuda")
    K = torch.zeros(36 * beam.nnzb, dtype=beam.k_dtype(precision), device="cuda")
    beam.assemble(_dev(u), precision, f, K)
    torch.cuda.synchronize()
    return f.cpu().numpy(), beam.to_csr(K)


@pytest.mark.parametrize("precision,tol", [(L.XK_FP64, TOL64), (L.XK_MIXED, TOLMIX)])
def test_beam_large_rotation_elements(precision, tol):
    z = golden("beam_elements")
    n = 6 * len(z["X"])
    f, K = _beam_eval(z["X"], z["conn"], z["u"], _sec(z), precision)
    assert rel_err(f, z["beam_f"]) < tol
    assert sparse_rel_err(K, golden_csr(z, "beam_K", n)) < tol
    f, K = _beam_eval(z["X"], z["conn"], z["u"], _sec(z, scf=0.25), precision, v_ref=[0.3, -0.2, 0.9])
    assert rel_err(f, z["beam_f_vref_scf"]) < tol
    assert sparse_rel_err(K, golden_csr(z, "beam_K_vref_scf", n)) < tol


@pytest.mark.parametrize("name", ["strand7", "strand19_slip"])
@pytest.mark.parametrize("precision,tol", [(L.XK_FP64, TOL64), (L.XK_MIXED, TOLMIX)])
def test_beam_strand(name, precision, tol):
    z = golden(name)
    n = 6 * len(z["X"])
    f, K = _beam_eval(z["X"], z["conn"], z["u0"], _sec(z), precision)
    # f_int of a near-straight strand is a small difference of large element forces:
    # compare against the element force scale
    fe, _ = ob.element_batch(z["X"], z["conn"], z["u0"], ob.Section(**_sec(z)), stiffness=False)
    assert np.max(np.abs(f - z["beam_f"])) < tol * np.max(np.abs(fe))
    assert sparse_rel_err(K, golden_csr(z, "beam_K", n)) < tol


def test_narrowphase_bit_exact():
    z = golden("narrowphase")
    N = len(z["s"])
    coords = np.concatenate([z["xA0"], z["xA1"], z["xB0"], z["xB1"]])
    idx = np.arange(N)
    conn = np.concatenate([np.stack([idx, N + idx], 1), np.stack([2 * N + idx, 3 * N + idx], 1)])
    mesh = DeviceMesh(coords, conn, 0.0)
    tab = oc.new_pairs(np.stack([idx, N + idx], 1), conn, np.zeros(2 * N))
    tab["normal"] = z["prev_n"].copy()
    tab["t1"] = z["prev_t1"].copy()
    pt = DevicePairTable(mesh.device)
    pt.from_host(tab)
    cp = L.ContactParams(1.0, 0.5, 0.1, 0.0, 0.0, 1e-6, 1)
    import ctypes as C
    L.call("xk_narrowphase", C.byref(mesh.c), C.byref(pt.c), C.c_void_p(_dev(np.zeros(6 * 4 * N)).data_ptr()),
           C.byref(cp), 0, C.c_void_p(torch.cuda.current_stream().cuda_stream))
    h = pt.to_host()
    assert np.array_equal(h["s"], z["s"]) and np.array_equal(h["t"], z["t"])
    assert np.array_equal(h["gap"], z["dist"])
    assert np.array_equal(h["normal"], z["n"])
    assert np.array_equal(h["t1"], z["t1"]) and np.array_equal(h["t2"], z["t2"])


def _engine_for(z, precision="fp64"):
    X, conn = z["X"], z["conn"]
    return AssemblyEngine(X, conn, float(z["radius"]), _sec(z), layer=z["elem_layer"], precision=precision,
                          k_pen=float(z["k_pen"]), k_t_ratio=float(z["k_t_ratio"]), mu=float(z["mu"]),
                          smoothing_delta=float(z["smoothing_delta"]))


@pytest.mark.parametrize("name", ["strand7", "strand7_nogap", "strand19_slip"])
def test_strand_sequence_fp64(name):
    """Detect / active set / Newton iterations against the reference's own outputs."""
    z = golden(name)
    eng = _engine_for(z, "fp64")
    X, conn = z["X"], z["conn"]
    n = 6 * len(X)
    sec = ob.Section(**_sec(z))
    for inc in range(int(z["n_incr"])):
        u_ref = _dev(z[f"inc{inc}_u_ref"])
        st = eng.detect(_dev(z[f"inc{inc}_u"]))
        assert st["candidates"] == len(z[f"inc{inc}_candidates"])
        h = eng.pair_state()
        p = f"inc{inc}_geom_"
        assert np.array_equal(h["ea"], z[p + "ea"]) and np.array_equal(h["eb"], z[p + "eb"])
        assert np.array_equal(h["status"], z[p + "status"])
        assert np.array_equal(h["gap"], z[p + "gap"])
        for it in range(int(z["n_iter"])):
            p = f"inc{inc}_it{it}_"
            u = z[p + "u"]
            eng.assemble(_dev(u), u_ref)
            torch.cuda.synchronize()
            h = eng.pair_state()
            assert np.array_equal(h["status"], z[p + "status"])
            assert np.array_equal(h["stick"], z[p + "stick"])
            for k in ("p_n", "z_t", "q_trial_norm", "k_t"):
                assert rel_err(h[k], z[p + k]) < TOL64, k
            Kb, fb = ob.assemble_beam(X, conn, u, sec)
            R_exp = fb - (z[p + "f_n"] + z[p + "f_f"])
            assert rel_err(eng.R.cpu().numpy(), R_exp) < TOL64
            Kc_exp = (golden_csr(z, p + "K_n", n) - golden_csr(z, p + "K_f", n)).tocsr()
            assert sparse_rel_err(eng.K_contact_csr(), Kc_exp) < TOL64
            assert sparse_rel_err(eng.K_beam_csr(), Kb) < TOL64
            assert abs(eng.residual_norm() - np.linalg.norm(R_exp)) <= TOL64 * np.linalg.norm(R_exp) + 1e-300


def test_strand_sequence_mixed():
    z = golden("strand19_slip")
    e64, emx = _engine_for(z, "fp64"), _engine_for(z, "mixed")
    for inc in range(int(z["n_incr"])):
        u0 = _dev(z[f"inc{inc}_u"])
        u_ref = _dev(z[f"inc{inc}_u_ref"])
        s64, smx = e64.detect(u0), emx.detect(u0)
        s64.pop("narrowphase_exact")
        smx.pop("narrowphase_exact")
        assert s64 == smx  # the same candidates, pairs and active set in both modes
        for it in range(int(z["n_iter"])):
            u = _dev(z[f"inc{inc}_it{it}_u"])
            e64.assemble(u, u_ref)
            emx.assemble(u, u_ref)
            torch.cuda.synchronize()
            fc64 = e64.R.cpu().numpy()
            fcmx = emx.R.cpu().numpy()
            assert rel_err(fcmx, fc64) < TOLMIX
            assert sparse_rel_err(emx.K_contact_csr(), e64.K_contact_csr()) < TOLMIX
            assert sparse_rel_err(emx.K_beam_csr(), e64.K_beam_csr()) < TOLMIX
            h64, hmx = e64.pair_state(), emx.pair_state()
            assert np.array_equal(h64["status"], hmx["status"])


@pytest.mark.parametrize("cfg", ["strand37"])
def test_engine_vs_oracle_medium(cfg):
    """37-wire strand (4,736 elements, ~30k pairs): GPU against the oracle on the same inputs."""
    from xkgpu import workloads as W

    w = W.config_workload(cfg, seed=1)
    st = w.strand
    eng = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision="fp64", **w.engine_kwargs())
    n = st.ndof
    u = w.u
    stats = eng.detect(_dev(u))
    table, cands, raw = oc.detect(oc.empty_table(), oc.deformed_coords(st.coords, u), st.conn, st.radii,
                                  elem_layer=st.elem_layer, exclude_same_layer=True)
    assert stats["raw"] == len(raw)
    assert stats["candidates"] == len(cands)
    table = oc.update_geometry(table, oc.deformed_coords(st.coords, u))
    h = eng.pair_state()
    assert np.array_equal(h["ea"], table["ea"]) and np.array_equal(h["eb"], table["eb"])
    assert np.array_equal(h["status"], table["status"])
    rng = np.random.default_rng(3)
    u_ref = u.copy()
    for it in range(2):
        u = u + rng.normal(0.0, 3e-4 * w.meta["d"], n) * np.tile([1, 1, 1, 0, 0, 0], st.n_nodes)
        eng.assemble(_dev(u), _dev(u_ref))
        torch.cuda.synchronize()
        table, fc, Kc, _ = oc.contact_iteration(table, st.coords, u, u_ref, n, k_pen=w.k_pen, k_t_ratio=w.k_t_ratio,
                                                mu_eff=w.mu)
        Kb, fb = ob.assemble_beam(st.coords, st.conn, u, ob.Section(**w.section, scf=None))
        h = eng.pair_state()
        assert np.array_equal(h["status"], table["status"])
        assert np.array_equal(h["stick"], table["stick"])
        assert rel_err(eng.R.cpu().numpy(), fb + fc) < TOL64
        assert sparse_rel_err(eng.K_contact_csr(), Kc) < TOL64
        assert sparse_rel_err(eng.K_beam_csr(), Kb) < TOL64


def test_graph_replay_matches_eager():
    z = golden("strand7")
    a, b = _engine_for(z), _engine_for(z)
    u0 = _dev(z["inc0_u"])
    a.detect(u0)
    b.detect(u0)
    u = _dev(z["inc0_it0_u"])
    u_ref = _dev(z["inc0_u_ref"])
    a.assemble(u, u_ref)
    b.capture(u, u_ref)  # warm-up + capture: runs assemble once
    torch.cuda.synchronize()
    assert torch.equal(a.R, b.R)
    a.gather_variant = b.gather_variant  # the tangent schedule the capture's autotuner chose
    a.assemble(u, u_ref)
    b.replay()
    torch.cuda.synchronize()
    assert torch.equal(a.R, b.R) and torch.equal(a.K_c, b.K_c) and torch.equal(a.K_beam, b.K_beam)


def test_deterministic_repeat():
    from xkgpu import workloads as W

    w = W.config_workload("strand37", seed=2)
    st = w.strand
    outs = []
    for _ in range(2):
        eng = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision="mixed", **w.engine_kwargs())
        eng.detect(_dev(w.u))
        eng.assemble(_dev(w.u * 1.01), _dev(w.u))
        torch.cuda.synchronize()
        outs.append((eng.R.clone(), eng.K_c[: 9 * eng.pattern.nnzb].clone(), eng.K_beam.clone()))
    for x, y in zip(outs[0], outs[1]):
        assert torch.equal(x, y)


@pytest.mark.parametrize("scf,v_ref,key", [(None, None, "beam_f"), (0.25, [0.3, -0.2, 0.9], "beam_f_vref_scf")])
def test_beam_float_path_large_rotations(scf, v_ref, key):
    """The all-float mixed beam kernel (cancellation-free frame) on rotations up to 1.5 rad."""
    z = golden("beam_elements")
    n = 6 * len(z["X"])
    eng = AssemblyEngine(z["X"], z["conn"], 0.0, _sec(z, scf=scf), precision="mixed", k_pen=1.0, v_ref=v_ref)
    eng.assemble(_dev(z["u"]))
    torch.cuda.synchronize()
    kkey = "beam_K" if key == "beam_f" else "beam_K_vref_scf"
    assert rel_err(eng.f_int.cpu().numpy(), z[key]) < TOLMIX
    assert sparse_rel_err(eng.K_beam_csr(), golden_csr(z, kkey, n)) < TOLMIX


def test_beam_float_chain_launch_equals_colours():
    """The one-launch float beam of wire meshes gives the same bits as the colour launches (store,
    then add): the ordered form (each shared node's two contributions summed by the lane that owns
    the node, one writer per block) and the atomic form (node rows and diagonal blocks zeroed, then
    two atomic adds); every shared value is one order-free sum of two terms."""
    import ctypes as C

    from xkgpu import workloads as W
    from xkgpu.device import ptr, stream_handle

    w = W.config_workload("strand37", seed=3)
    st = w.strand
    eng = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision="mixed", **w.engine_kwargs())
    assert eng.beam.node_diag is not None and eng.beam.chain_ordered  # wires are chains, in order
    u0 = _dev(w.u)
    eng.detect(u0)
    eng.assemble(u0 * 1.001, u0)
    colours = DeviceBeam(eng.mesh, w.section, chain=False)
    assert colours.node_diag is None and colours.plan.n_colors >= 2
    atomic = DeviceBeam(eng.mesh, w.section)
    atomic.plan.chain_ordered = 0
    for beam in (colours, atomic):
        f = torch.full_like(eng.f_int, float("nan"))
        K = torch.full_like(eng.K_beam, float("nan"))
        L.call("xk_beam_assemble32", C.byref(eng.mesh.c), C.byref(beam.section), ptr(eng.elem32),
               C.byref(beam.plan), ptr(eng.node32), ptr(f), ptr(K), stream_handle(None))
        torch.cuda.synchronize()
        assert torch.equal(f, eng.f_int)
        assert torch.equal(K[: 36 * beam.nnzb], eng.K_beam[: 36 * beam.nnzb])


def test_beam_float_capped_launch_loops_to_the_same_bits():
    """The float beam launch capped at one CTA per SM loops over its work (strand397: 38,112 elements,
    about twice the capped grid) and gives the bits of the full grid, ordered and colour forms."""
    import ctypes as C

    from xkgpu import workloads as W
    from xkgpu.device import ptr, stream_handle

    w = W.config_workload("strand397", seed=1)
    st = w.strand
    eng = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision="mixed", **w.engine_kwargs())
    u0 = _dev(w.u)
    eng.assemble(u0 * 1.001, u0)  # node records, element records, the ordered full-grid launch
    torch.cuda.synchronize()
    capped = DeviceBeam(eng.mesh, w.section)
    capped.plan.beam_ctas_per_sm = 1
    colours = DeviceBeam(eng.mesh, w.section, chain=False)
    capped_colours = DeviceBeam(eng.mesh, w.section, chain=False)
    capped_colours.plan.beam_ctas_per_sm = 1
    assert 32 * (st.n_elems // 31 + 1) > 128 * 152  # the capped ordered launch loops
    for beam in (capped, colours, capped_colours):
        f = torch.full_like(eng.f_int, float("nan"))
        K = torch.full_like(eng.K_beam, float("nan"))
        L.call("xk_beam_assemble32", C.byref(eng.mesh.c), C.byref(beam.section), ptr(eng.elem32),
               C.byref(beam.plan), ptr(eng.node32), ptr(f), ptr(K), stream_handle(None))
        torch.cuda.synchronize()
        assert torch.equal(f, eng.f_int)
        assert torch.equal(K[: 36 * beam.nnzb], eng.K_beam[: 36 * beam.nnzb])


def test_beam_float_ordered_writes_every_block_once():
    """The ordered float beam writes every f row and stored block of the mesh (buffers start as NaN),
    on meshes whose wires end inside a warp's range, at a warp boundary, and as one-element wires."""
    import ctypes as C

    from xkgpu.device import ptr, stream_handle

    z = golden("beam_elements")
    sec = _sec(z)
    for lengths in ([31, 31, 1, 5, 62, 2], [1] * 40, [64, 30, 33]):
        coords, conn, n0 = [], [], 0
        for k, n_el in enumerate(lengths):
            xs = np.linspace(0.0, 2.0 * n_el, n_el + 1)
            coords.append(np.stack([xs, 0 * xs + 3.0 * k, 0 * xs], 1))
            conn.append(np.stack([n0 + np.arange(n_el), n0 + np.arange(1, n_el + 1)], 1))
            n0 += n_el + 1
        X, cn = np.concatenate(coords), np.concatenate(conn)
        rng = np.random.default_rng(len(lengths))
        u = np.concatenate([1e-2 * rng.normal(size=(len(X), 3)), 0.3 * rng.normal(size=(len(X), 3))], 1).ravel()
        eng = AssemblyEngine(X, cn, 0.25, sec, precision="mixed", k_pen=1.0)
        assert eng.beam.chain_ordered
        eng.f_int.fill_(float("nan"))
        eng.K_beam.fill_(float("nan"))
        eng.assemble(_dev(u))
        torch.cuda.synchronize()
        assert torch.isfinite(eng.f_int).all()
        assert torch.isfinite(eng.K_beam[: 36 * eng.beam.nnzb]).all()
        colours = DeviceBeam(eng.mesh, sec, chain=False)
        f = torch.zeros_like(eng.f_int)
        K = torch.zeros_like(eng.K_beam)
        L.call("xk_beam_assemble32", C.byref(eng.mesh.c), C.byref(colours.section), ptr(eng.elem32),
               C.byref(colours.plan), ptr(eng.node32), ptr(f), ptr(K), stream_handle(None))
        torch.cuda.synchronize()
        assert torch.equal(f, eng.f_int)
        assert torch.equal(K[: 36 * colours.nnzb], eng.K_beam[: 36 * colours.nnzb])
        Kref, fref = ob.assemble_beam(X, cn, u, ob.Section(**{**sec, "scf": None}))
        assert rel_err(eng.f_int.cpu().numpy(), fref) < TOLMIX
        assert sparse_rel_err(eng.K_beam_csr(), Kref) < TOLMIX


def test_near_parallel_pairs_mixed_vs_fp64():
    """Pairs of (near-)parallel segments, which the float pair kernels hand to their exact-routine
    kernels: touching parallel wires (members), a wire at 1 degree to them and one parallel just
    out of contact (other pairs), plus a crossing wire; mixed against FP64."""
    n_el, r = 8, 1.0
    xs = np.linspace(0.0, 16.0, n_el + 1)
    ang = np.deg2rad(1.0)
    wires = [
        np.stack([xs, 0 * xs, 0 * xs], 1),
        np.stack([xs, 0 * xs + 2 * r * (1 - 2e-3), 0 * xs], 1),  # parallel, in contact
        np.stack([xs, 0 * xs - 2 * r * (1 + 1e-4), 0 * xs], 1),  # parallel, just apart
        np.stack([xs * np.cos(ang), xs * np.sin(ang) - 2 * r * (1 - 1e-3), 0 * xs + 0.05], 1) + [0.0, 0.0, 0.0],
        np.stack([8.0 + 0 * xs, xs - 8.0, 0 * xs + 2 * r * (1 - 2e-3)], 1),  # crossing
    ]
    coords = np.concatenate(wires)
    conn = np.concatenate([np.stack([np.arange(n_el), np.arange(1, n_el + 1)], 1) + k * (n_el + 1)
                           for k in range(len(wires))]).astype(np.int64)
    layer = np.repeat(np.arange(len(wires)), n_el)
    sec = {"E": 2.0e5, "G": 2.0e5 / 2.6, "A": np.pi, "Iy": np.pi / 4, "Iz": np.pi / 4, "J": np.pi / 2,
           "kappa_y": 0.886, "kappa_z": 0.886, "scf": None}
    rng = np.random.default_rng(7)
    u = np.zeros(6 * coords.shape[0])
    u.reshape(-1, 6)[:, :3] = rng.normal(0.0, 1e-4, (coords.shape[0], 3))
    out = {}
    for prec in ("fp64", "mixed"):
        eng = AssemblyEngine(coords, conn, r, sec, layer=layer, precision=prec, k_pen=1e4, mu=0.2, margin=0.05)
        u0 = _dev(u)
        stats = eng.detect(u0)
        eng.assemble(u0 * 1.01, u0)
        eng.assemble(u0 * 1.02, u0)
        torch.cuda.synchronize()
        out[prec] = (eng.R.cpu().numpy(), eng.K_contact_csr(), eng.pair_state(), stats)
    R64, K64, h64, st64 = out["fp64"]
    Rmx, Kmx, hmx, stmx = out["mixed"]
    st64.pop("narrowphase_exact")
    stmx.pop("narrowphase_exact")  # how many pairs the mixed detection took through the exact routine
    assert st64 == stmx and st64["members"] > 0 and st64["pairs"] > st64["members"]
    assert rel_err(Rmx, R64) < TOLMIX
    assert sparse_rel_err(Kmx, K64) < TOLMIX
    assert np.array_equal(h64["status"], hmx["status"])
    assert rel_err(hmx["gap"], h64["gap"]) < 1e-6
    assert rel_err(hmx["s"], h64["s"]) < 1e-5 and rel_err(hmx["t"], h64["t"]) < 1e-5


@pytest.mark.parametrize("precision,tol", [("fp64", TOL64), ("mixed", TOLMIX)])
def test_engine_coated_wires_vs_oracle(precision, tol):
    """The coating model fused into the pair kernels (7-wire strand, coating 0.1 r): detection with the
    core gap, coating compression and the coating term of the active set, then two Newton iterations
    whose residual and K_c carry the Huber, friction, coating and coating-friction parts; against the
    oracle (which matches the reference's own outputs on these inputs, tests/golden/coating7.npz)."""
    from xkgpu import workloads as W

    z = golden("coating7")
    X, conn, layer = z["X"], z["conn"], z["elem_layer"]
    n = 6 * len(X)
    r, cr = float(z["radius"]), float(z["core_radius"])
    k, c, cmu, ktr, dt = (float(z[q]) for q in ("k_coat", "c_coat", "mu_coat", "kt_ratio", "dt"))
    sec = W.circle_section(2.0 * r)
    k_pen, mu, kt_ratio = 2e4, 0.1, 0.5
    eng = AssemblyEngine(X, conn, r, sec, layer=layer, precision=precision, k_pen=k_pen, k_t_ratio=kt_ratio, mu=mu,
                         core_radii=cr, coating=dict(stiffness=k, damping=c, mu=cmu, k_t_ratio=ktr, dt=dt))
    u0 = z["u0"]
    eng.detect(_dev(u0))
    table, _, _ = oc.detect(oc.empty_table(), oc.deformed_coords(X, u0), conn, np.full(len(conn), r),
                            elem_layer=layer, exclude_same_layer=True, core_radii=np.full(len(conn), cr))
    table, cc = oc.coating_geometry(table, oc.deformed_coords(X, u0))
    h = eng.pair_state()
    assert np.array_equal(h["ea"], table["ea"]) and np.array_equal(h["status"], table["status"])
    if precision == "fp64":  # the detection is exact in both modes; the mixed state is read back as float
        assert np.array_equal(h["gap"], table["gap"]) and np.array_equal(h["coat_cc"], cc)
    else:
        assert rel_err(h["gap"], table["gap"]) < 1e-6 and rel_err(h["coat_cc"], cc) < 1e-6
    assert eng.pattern.n_members == len(cc)  # every pair of a coated model contributes
    eng.end_step()  # coating_compression_prev <- coating_compression
    cc_prev = cc.copy()
    state = {"z_t": np.zeros((len(cc), 2)), "stick": np.ones(len(cc), bool), "q_trial_norm": np.zeros(len(cc)),
             "dissipation": np.zeros(len(cc))}
    sec_o = ob.Section(**sec, scf=None)
    for it in range(int(z["n_iter"])):
        u = z[f"it{it}_u"]
        eng.assemble(_dev(u), _dev(u0))
        torch.cuda.synchronize()
        cd = oc.deformed_coords(X, u)
        table, cc = oc.coating_geometry(table, cd, freeze_active_set=True)
        table, fn, _ = oc.huber_evaluate(table, n, k_pen)
        table, ff, _, fr = oc.friction_evaluate(table, u, u0, n, k_pen, kt_ratio, mu)
        fcn = oc.coating_forces(table, cc, cc_prev, n, k, c, dt)
        fcf, state = oc.coating_friction(table, cc, state, u, u0, n, k, ktr, cmu)
        Kb, fb = ob.assemble_beam(X, conn, u, sec_o)
        R_ref = fb - (fn + ff + fcn + fcf)
        K_ref = (oc.huber_tangent(table, n, k_pen) - oc.friction_tangent(table, fr, n)
                 + oc.coating_stiffness(table, cc, n, k, c, dt)
                 + oc.coating_friction_stiffness(table, cc, state, n, k, ktr, cmu)).tocsr()
        assert rel_err(eng.R.cpu().numpy(), R_ref) < tol, it
        assert sparse_rel_err(eng.K_contact_csr(), K_ref) < tol, it
        h = eng.pair_state()
        assert rel_err(h["coat_cc"], cc) < (1e-12 if precision == "fp64" else 1e-5)
        assert np.array_equal(h["coat_stick"], state["stick"])
        assert rel_err(h["coat_z_t"], state["z_t"]) < (1e-10 if precision == "fp64" else 1e-4)


def test_mixed_engine_vs_fp64_strand37():
    from xkgpu import workloads as W

    w = W.config_workload("strand37", seed=4)
    st = w.strand
    e64 = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision="fp64", **w.engine_kwargs())
    emx = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision="mixed", **w.engine_kwargs())
    u0 = _dev(w.u)
    s64, smx = e64.detect(u0), emx.detect(u0)
    s64.pop("narrowphase_exact")
    smx.pop("narrowphase_exact")
    assert s64 == smx
    rng = np.random.default_rng(9)
    for _ in range(3):
        du = rng.normal(0.0, 2e-4 * w.meta["d"], st.ndof) * np.tile([1, 1, 1, 1e-1, 1e-1, 1e-1], st.n_nodes)
        u = u0 + _dev(du)
        e64.assemble(u, u0)
        emx.assemble(u, u0)
        torch.cuda.synchronize()
        assert rel_err(emx.R.cpu().numpy(), e64.R.cpu().numpy()) < TOLMIX
        assert sparse_rel_err(emx.K_contact_csr(), e64.K_contact_csr()) < TOLMIX
        assert sparse_rel_err(emx.K_beam_csr(), e64.K_beam_csr()) < TOLMIX
        h64, hmx = e64.pair_state(), emx.pair_state()
        assert np.array_equal(h64["status"], hmx["status"])
        assert rel_err(hmx["gap"], h64["gap"]) < 1e-6


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("workload", ["strand7", "strand37"])
def test_tangent_gather_schedules_agree(precision, workload):
    """The contact-tangent reduction schedules give the same K_c, each deterministically; the residual
    from the element-side schedule's force sums equals the one gathered from the member records."""
    import ctypes as C

    from xkgpu import workloads as W
    from xkgpu.device import ptr, stream_handle

    w = W.config_workload(workload, seed=5)
    st = w.strand
    eng = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision=precision, **w.engine_kwargs())
    u0 = _dev(w.u)
    eng.detect(u0)
    eng.assemble(u0 * 1.001, u0)
    nb = eng.pattern.nnzb
    outs = []
    for v in (L.XK_GATHER_LANES, L.XK_GATHER_CHUNKS, L.XK_GATHER_LANES, L.XK_GATHER_SIDES, L.XK_GATHER_SIDES):
        K = torch.zeros_like(eng.K_c)
        L.call("xk_contact_gather_tangent", C.byref(eng.pattern.c), ptr(eng.rec), eng.precision, L.XK_OUT_COMBINED,
               L.XK_WHICH_COMBINED, v, ptr(K), stream_handle(None))
        torch.cuda.synchronize()
        outs.append(K[: 9 * nb].double().cpu().numpy())
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert rel_err(outs[1], outs[0]) < tol
    assert rel_err(outs[3], outs[0]) < tol
    assert np.array_equal(outs[0], outs[2])
    assert np.array_equal(outs[3], outs[4])
    # the residual from the element force sums left by the last gather equals the member-record gather
    R = {}
    for name in ("records", "elem_sums"):
        out = torch.zeros_like(eng.R)
        n2 = torch.zeros(1, dtype=torch.float64, device="cuda")
        if name == "records":
            L.call("xk_contact_gather_force", C.byref(eng.pattern.c), ptr(eng.rec), eng.precision,
                   L.XK_OUT_COMBINED, L.XK_WHICH_COMBINED, ptr(eng.f_int), -1.0, None, None, ptr(out), ptr(n2),
                   stream_handle(None))
        else:
            L.call("xk_contact_gather_force_elem", C.byref(eng.pattern.c), eng.precision, ptr(eng.f_int), -1.0,
                   None, None, ptr(out), ptr(n2), stream_handle(None))
        torch.cuda.synchronize()
        R[name] = (out.cpu().numpy(), float(n2.item()))
    assert rel_err(R["elem_sums"][0], R["records"][0]) < (1e-12 if precision == "fp64" else 1e-6)
    assert abs(R["elem_sums"][1] - np.sum(R["elem_sums"][0] ** 2)) <= 1e-12 * R["elem_sums"][1]


def test_host_pipeline_returns_each_steps_outputs():
    """Pipelined host round trips: every ticket holds its own step's R, K_beam and K_c."""
    from xkgpu import workloads as W
    from xkgpu.engine import HostPipeline

    w = W.config_workload("strand37", seed=4)
    st = w.strand
    kw = w.engine_kwargs()
    kw["mu"] = 0.0  # no friction history: every step's outputs depend on its own inputs only
    ref = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision="mixed", **kw)
    eng = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision="mixed", **kw)
    u0 = _dev(w.u)
    ref.detect(u0)
    eng.detect(u0)
    rng = np.random.default_rng(8)
    mask = np.tile([1, 1, 1, 0, 0, 0], st.n_nodes)
    us = [w.u + rng.normal(0.0, 1e-3 * w.meta["d"], w.u.shape) * mask for _ in range(3)]
    pipe = HostPipeline(eng)
    ref.gather_variant = eng.gather_variant
    hosts = [torch.as_tensor(x).pin_memory() for x in us]
    uref_h = torch.as_tensor(w.u).pin_memory()

    def check(ticket, i):
        R, Kb, Kc = pipe.result(ticket)
        ref.assemble(_dev(us[i]), u0)
        assert torch.equal(R, ref.R.cpu())
        assert torch.equal(Kb, ref.K_beam.cpu())
        assert torch.equal(Kc, ref.K_c[: Kc.numel()].cpu())
        # the full matrices rebuilt from the host copies equal the engine's own views
        assert (eng.K_beam_csr(Kb) != ref.K_beam_csr()).nnz == 0
        assert (eng.K_contact_csr(Kc) != ref.K_contact_csr()).nnz == 0

    # the usual loop: submit step k, then read step k-1 while step k runs
    prev = pipe.submit(hosts[0], uref_h)
    for k in range(1, 5):
        cur = pipe.submit(hosts[k % 3], uref_h)
        check(prev, (k - 1) % 3)
        prev = cur
    check(prev, 4 % 3)
    # R and its squared norm only (a device linear solve keeps the tangent on the GPU)
    del pipe
    lean = HostPipeline(eng, read_tangent=False)
    assert lean.bytes_out == 8 * (6 * st.n_nodes + 1)
    prev = lean.submit(hosts[0], uref_h)
    for k in range(1, 4):
        cur = lean.submit(hosts[k % 3], uref_h)
        R, Kb, Kc = lean.result(prev)
        ref.assemble(_dev(us[(k - 1) % 3]), u0)
        assert Kb is None and Kc is None
        assert torch.equal(R, ref.R.cpu())
        assert lean.residual_norm2() == float(ref.norm2.item())
        prev = cur


def test_conversions_in_integer_arithmetic_are_ieee():
    """The node records and the float copy of the pair table (and the way back) convert between
    double and float in integer arithmetic; their bits equal the IEEE conversions (torch's own
    .float() / .double() on the GPU), zeros and signs included."""
    import ctypes as C

    from xkgpu import workloads as W
    from xkgpu.device import ptr, stream_handle

    w = W.config_workload("strand37", seed=5)
    st = w.strand
    eng = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision="mixed", **w.engine_kwargs())
    u0 = _dev(w.u)
    rng = np.random.default_rng(3)
    u1 = _dev(w.u + rng.normal(0.0, 1e-3, w.u.shape))
    # node records: x = X + u split into float hi / lo, u and u - u_ref in float
    L.call("xk_nodes_prepare", C.byref(eng.mesh.c), ptr(u1), ptr(u0), ptr(eng.node32), stream_handle(None))
    torch.cuda.synchronize()
    N = eng.node32.view(-1, L.NODE32_STRIDE)[: st.n_nodes]
    x = eng.mesh.X.view(-1, 3) + u1.view(-1, 6)[:, :3]
    hi = x.float()
    assert torch.equal(N[:, 0:3], hi)
    assert torch.equal(N[:, 3:6], (x - hi.double()).float())
    assert torch.equal(N[:, 6:12], u1.view(-1, 6).float())
    assert torch.equal(N[:, 12:15], (u1 - u0).view(-1, 6)[:, :3].float())
    # the pair table: a detection ends with the float copy, the way back must return the float values;
    # an assembly between two detections gives the pairs their contact state (p_n, z_t, k_pen)
    eng.detect(u0)
    eng.assemble(u1, u0)
    eng.detect(u1)
    n, cap = eng.pairs.n, eng.pairs.cap
    t = eng.pairs.t
    fields = {"s": 1, "t": 1, "gap": 1, "normal": 3, "t1": 3, "t2": 3, "p_n": 1, "z_t": 2, "q_trial_norm": 1,
              "dissipation": 1, "k_pen": 1, "k_t": 1}
    before = {k: torch.stack([t[k][c * cap: c * cap + n] for c in range(w_)]).clone() for k, w_ in fields.items()}
    assert bool((before["p_n"] != 0).any()) and bool((before["gap"] < 0).any())  # a contact state, not zeros only
    eng.sync_state()
    torch.cuda.synchronize()
    others = torch.zeros(n, dtype=torch.bool, device=u0.device)
    pat = eng.pattern
    others[eng.pairs32.t["pair"][pat.n_members: n].long()] = True
    for k, w_ in fields.items():
        after = torch.stack([t[k][c * cap: c * cap + n] for c in range(w_)])
        exp = before[k].float().double()
        if k == "t2":  # the other pairs' t2 is formed again as n x t1
            after, exp = after[:, ~others], exp[:, ~others]
        assert torch.equal(after, exp), k
        assert torch.equal(torch.signbit(after), torch.signbit(exp)), k
