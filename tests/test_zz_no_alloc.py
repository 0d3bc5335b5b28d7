"""xk_constraint_jacobian_noalloc: the allocation-free constraint Jacobian.

It must give what xk_constraint_jacobian gives on the same pair table, on two
calls in a row (the second one reuses the static scratch that the first one
left behind), and refuse tables beyond its stated maximum before touching the
device.  Compared bit for bit: both run the same kernels.  The device's default
memory pool (which the allocating entry point's stream-ordered allocations
come from) shows no allocation during a no-alloc call, while it does show the
allocating entry point's scratch.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from xkgpu import _lib as L  # noqa: E402


def test_noalloc_rejects_oversized_table():
    """The size check comes first; no device is needed to see the error."""
    L.load()
    mesh = L.Mesh()
    pairs = L.Pairs()
    pairs.n = L.JACOBIAN_NOALLOC_MAX_PAIRS + 1
    n_rows = C.c_int64(-1)
    code = L.call("xk_constraint_jacobian_noalloc", C.byref(mesh), C.byref(pairs), None, None, None, None, 0,
                  C.byref(n_rows), None, allow=(L.XK_ERR_ARG,))
    assert code == L.XK_ERR_ARG
    assert n_rows.value == 0
    assert b"XK_JACOBIAN_NOALLOC_MAX_PAIRS" in L.load().xk_last_error()


def _jacobian(name, eng, cap):
    from xkgpu.device import ptr, stream_handle

    dev = eng.device
    rows = torch.full((12 * cap,), -1, dtype=torch.int32, device=dev)
    cols = torch.full((12 * cap,), -1, dtype=torch.int32, device=dev)
    vals = torch.full((12 * cap,), np.nan, dtype=torch.float64, device=dev)
    pidx = torch.full((cap,), -1, dtype=torch.int32, device=dev)
    n_rows = C.c_int64(-1)
    L.call(name, C.byref(eng.mesh.c), C.byref(eng.pairs.c), ptr(rows), ptr(cols), ptr(vals), ptr(pidx), cap,
           C.byref(n_rows), stream_handle(None))
    torch.cuda.synchronize()
    n = n_rows.value
    return (n, rows[: 12 * n].cpu().numpy(), cols[: 12 * n].cpu().numpy(), vals[: 12 * n].cpu().numpy(),
            pidx[:n].cpu().numpy())


class _DefaultPool:
    """High-water mark of the current device's default memory pool (driver API through ctypes)."""

    RESERVED_MEM_CURRENT, USED_MEM_CURRENT, USED_MEM_HIGH = 5, 7, 8

    def __init__(self):
        self.cu = C.CDLL("libcuda.so.1")
        assert self.cu.cuInit(0) == 0
        dev = C.c_int(0)
        assert self.cu.cuDeviceGet(C.byref(dev), torch.cuda.current_device()) == 0
        self.pool = C.c_void_p()
        assert self.cu.cuDeviceGetDefaultMemPool(C.byref(self.pool), dev) == 0

    def get(self, attr) -> int:
        v = C.c_uint64(0)
        assert self.cu.cuMemPoolGetAttribute(self.pool, attr, C.byref(v)) == 0
        return v.value

    def reset_high(self):
        zero = C.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, self.USED_MEM_HIGH, C.byref(zero)) == 0

    def peak_during(self, fn) -> tuple[int, int]:
        """(bytes in use at the peak above the level before, change of the reserved bytes) over fn()."""
        torch.cuda.synchronize()
        self.reset_high()
        used0, res0 = self.get(self.USED_MEM_CURRENT), self.get(self.RESERVED_MEM_CURRENT)
        fn()
        torch.cuda.synchronize()
        return self.get(self.USED_MEM_HIGH) - used0, self.get(self.RESERVED_MEM_CURRENT) - res0


@pytest.mark.gpu
def test_noalloc_jacobian_matches_allocating_entry_point():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from xkgpu import workloads as W
    from xkgpu.engine import AssemblyEngine

    w = W.config_workload("strand37", seed=11)
    st = w.strand
    eng = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision="fp64", **w.engine_kwargs())
    u = torch.as_tensor(np.ascontiguousarray(w.u), dtype=torch.float64, device="cuda")
    eng.detect(u)
    eng.assemble(u, u)
    assert 0 < eng.pairs.n <= L.JACOBIAN_NOALLOC_MAX_PAIRS
    cap = eng.pairs.n

    ref = _jacobian("xk_constraint_jacobian", eng, cap)
    assert ref[0] > 0
    for _ in range(2):
        got = _jacobian("xk_constraint_jacobian_noalloc", eng, cap)
        assert got[0] == ref[0]
        for a, b in zip(got[1:], ref[1:]):
            assert np.array_equal(a, b)

    # no device allocation in a no-alloc call (after the first, set-up call above); the same
    # measurement sees the allocating entry point's per-pair flags
    from xkgpu.device import ptr, stream_handle

    pool = _DefaultPool()
    out = [torch.empty(12 * cap, dtype=t, device="cuda") for t in (torch.int32, torch.int32, torch.float64)]
    pidx = torch.empty(cap, dtype=torch.int32, device="cuda")

    def call(name):
        n_rows = C.c_int64(-1)
        L.call(name, C.byref(eng.mesh.c), C.byref(eng.pairs.c), *(ptr(t) for t in out), ptr(pidx), cap,
               C.byref(n_rows), stream_handle(None))
        assert n_rows.value == ref[0]

    peak, reserved = pool.peak_during(lambda: call("xk_constraint_jacobian"))
    assert peak >= 4 * cap
    peak, reserved = pool.peak_during(lambda: call("xk_constraint_jacobian_noalloc"))
    assert (peak, reserved) == (0, 0)

    # the same rows as the oracle's constraint Jacobian
    from oracle import contact as oc

    import scipy.sparse as sp

    host = eng.pairs.to_host()
    conn = np.asarray(st.conn, dtype=np.int64)
    host["nodes"] = np.concatenate([conn[host["ea"]], conn[host["eb"]]], axis=1)
    G, act = oc.constraint_jacobian(host, eng.mesh.ndof)
    assert list(ref[4]) == act
    n = ref[0]
    Gd = sp.csr_matrix((ref[3], (ref[1], ref[2])), shape=(n, eng.mesh.ndof))
    assert abs(Gd - G).max() <= 1e-12 * max(abs(G).max(), 1.0)
