"""Strand meshes generated on the GPU against the reference's meshes and the host generator."""

from __future__ import annotations

import warnings

import numpy as np
import pytest

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # collected on CPU-only hosts, skipped there
    pytest.skip("no CUDA device", allow_module_level=True)

from xkgpu import strand as S  # noqa: E402
from xkgpu import workloads as W  # noqa: E402


def test_device_strands_match_reference_meshes():
    """The reference generator's 7-, 19- and 37-wire meshes (golden fixtures), made on the device."""
    z = golden("meshes")
    warnings.simplefilter("ignore")
    for tag, args, kw in (("w7", (7, 2.0, 40.0, 1, 16), dict(gap=-0.01)),
                          ("w19", (19, 1.0, 20.0, 2, 32), dict(gap=0.0)),
                          ("w37", (37, 0.5, 20.0, 2, 48), dict(gap=-0.0025))):
        host = S.make_strand(*args, **kw)  # raises a non-negative gap to the minimum safe gap
        X, conn, layer, radii = S.generate_on_device([S.strand_spec(host)])
        torch.cuda.synchronize()
        assert np.array_equal(conn.cpu().numpy(), z[tag + "_conn"])
        # cos / sin of the device may differ from the host's libm in the last bit
        assert rel_err(X.cpu().numpy(), z[tag + "_X"]) < 1e-15
        wire_layer = np.asarray(z[tag + "_layer"])
        assert np.array_equal(layer.cpu().numpy(), np.repeat(wire_layer, host.n_elems_per_wire))
        assert np.array_equal(radii.cpu().numpy(), host.radii)


def test_device_batch_matches_host_merge():
    """Many strands of the batched workload (7/19/37 wires, coarse and fine pitches) in one launch."""
    rng = np.random.default_rng(3)
    strands = []
    warnings.simplefilter("ignore")
    for _ in range(24):
        nw = int(rng.choice([3, 7, 19, 37]))
        npt = int(rng.integers(1, 5))
        epp = int(rng.integers(8, 49))
        strands.append(S.make_strand(nw, 2.0, 40.0, npt, epp * npt, gap=-0.01, allow_coarse=True))
    merged, _, node_first = S.merge_strands(strands)
    offs = S.strand_offsets(strands)
    elem_first = np.concatenate([[0], np.cumsum([s.n_elems for s in strands])[:-1]])
    specs = [S.strand_spec(s, x_offset=o, node_first=int(n0), elem_first=int(e0))
             for s, o, n0, e0 in zip(strands, offs, node_first, elem_first)]
    X, conn, layer, radii = S.generate_on_device(specs)
    torch.cuda.synchronize()
    assert np.array_equal(conn.cpu().numpy(), merged.conn)
    assert np.array_equal(layer.cpu().numpy(), merged.elem_layer)
    assert np.array_equal(radii.cpu().numpy(), merged.radii)
    assert rel_err(X.cpu().numpy(), merged.coords) < 1e-15
    # the workload builder's batch is the same construction
    w = W.config_workload("batch8", seed=1)
    assert w.strand.n_nodes > 0
