"""The bending run of the 91-wire configuration (bend by prescribed end sections, release, free oscillation
under Generalized-alpha) on a 7-wire strand: FP64 and mixed through the reference's solver loop.

``xkgpu.runs.run_bend_oscillation`` bends the strand dynamically to an arc of curvature 1/(50 D) over
1 ms, releases the z = L ends and takes two Generalized-alpha steps of 1e-4 s.  The FP64 run must complete
(every increment of the bend and of the steps converged); the mixed run follows the FP64 run's increments
(``follow``) and must complete too, with displacements within 1e-6 of the FP64 run's, max-norm relative,
at every common increment and at the end of every step taken on the same increments.  Both runs use a
force tolerance of 1e-6 (the mixed residual's floor is near 1e-7 of an increment's first residual).
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from xkgpu import runs  # noqa: E402
from xkgpu import solver as S  # noqa: E402
from xkgpu import workloads as W  # noqa: E402


def test_bend_release_oscillation_fp64_and_mixed():
    w = W.strand_workload("strand7", 7, 2.0, 40.0, 1, 16, gap_frac=0.0, seed=0, penalty="beam_ei")
    D = 2.0 * max(x.lay_radius for x in w.strand.wires) + w.meta["d"]
    cfg = dict(dt_min_fraction=1e-3, max_nr_attempts=100, use_line_search=False, tol_force=1e-6)
    kw = dict(kappa=1.0 / (50.0 * D), n_steps=2, bend_time=1e-3, bend_settings=S.SolverSettings(dt_max_fraction=0.1, **cfg),
              step_settings=S.SolverSettings(**cfg))
    a = runs.run_bend_oscillation(w, "fp64", **kw)
    assert a["converged"], a["bend"]
    b = runs.run_bend_oscillation(w, "mixed", follow=a["schedule"], **kw)
    assert b["converged"], b["bend"]
    fa = {round(f, 12): k for k, f in enumerate(a["bend"]["load_frac"])}
    common = [(fa[round(f, 12)], k) for k, f in enumerate(b["bend"]["load_frac"]) if round(f, 12) in fa]
    assert len(common) == len(a["bend"]["load_frac"])  # every FP64 increment was also a mixed one
    for ka, kb in common:
        ua, ub = a["bend_u"][ka], b["bend_u"][kb]
        assert np.max(np.abs(ub - ua)) <= 1e-6 * np.max(np.abs(ua))
    assert len(a["u"]) == len(b["u"]) == 3  # the bent state and the two steps
    # the bent state, and every step taken on the same increments as the FP64 run's (a mixed cutback adds
    # increments, and the Generalized-alpha response then differs by its time discretisation)
    same = a["schedule"][0] == [f for f in b["schedule"][0] if round(f, 12) in fa]
    for k, (ua, ub) in enumerate(zip(a["u"], b["u"])):
        if k > 0:
            same = same and a["schedule"][k] == b["schedule"][k]
        if not same:
            break
        assert np.max(np.abs(ub - ua)) <= 1e-6 * np.max(np.abs(ua)), k
