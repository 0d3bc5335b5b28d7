"""Device-resident assembly of one Newton iteration of the strand contact solver.

Per increment (``detect``), as at the top of the reference's step loop
(``xkep_cae/contact/solver/process.py:406-429``):

1. broadphase + shared-node / same-layer / midpoint filters on X + u
   (``DetectCandidatesProcess``),
2. merge into the pair table (disappeared pairs turn INACTIVE),
3. exact narrowphase with the active-set update (``UpdateGeometryProcess``),
4. node incidence of the pairs that can contribute and the K_c block pattern.

Per Newton iteration (``assemble``), as ``ContactForceAssemblyProcess`` +
``TangentAssemblyProcess`` (``contact/solver/_newton_steps.py:79-135,289-313``):

1. fused pair kernel: frozen narrowphase, Huber normal force, Coulomb return
   mapping (state z_t <- q), factorised pair tangent,
2. beam f_int and K_T (coloured, atomic-free),
3. residual R = f_int - (f_n + f_f) - f_ext with R[fixed] = 0 and its FP64
   squared norm,
4. contact tangent K_c = K_n - K_f in 3x3 blocks.

``K_T = K_beam + K_c`` is kept as two block matrices on the device; scipy
views are built on request only.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import scipy.sparse as sp
import torch

from . import _lib as L
from .device import (DeviceBeam, DeviceContactPattern, DeviceMesh, DevicePairTable, DevicePairTable32, ptr,
                     require_cuda, stream_handle)

PRECISIONS = {"fp64": L.XK_FP64, "mixed": L.XK_MIXED}


class AssemblyEngine:
    def __init__(self, coords, conn, radii, section: dict, *, layer=None, precision: str = "fp64",
                 k_pen: float, k_t_ratio: float = 0.5, mu: float | np.ndarray = 0.1, smoothing_delta: float = 0.0,
                 g_on: float = 0.0, g_off: float = 1e-6, allow_deactivation: bool = True,
                 exclude_same_layer: bool = True, exclude_shared: bool = True, midpoint_prescreening: bool = True,
                 prescreening_margin: float = 0.0, margin: float = 0.0, v_ref=None, device=None,
                 core_radii=None, coating: dict | None = None):
        """``core_radii`` and ``coating`` (keys ``stiffness``, ``damping``, ``mu``, ``k_t_ratio``, ``dt``)
        switch on the coated-wire model of ``KelvinVoigtCoatingProcess``: the gap is taken between the
        cores and every pair's coating force and friction enter the records (the model is on when the
        coating stiffness is positive, as in the reference)."""
        self.device = require_cuda(device)
        mu_elem = None
        if np.ndim(mu) > 0:  # one friction coefficient per element (batched strands)
            mu_elem, mu = np.asarray(mu, dtype=np.float64), 0.0
        co = dict(coating or {})
        self.coated = float(co.get("stiffness", 0.0)) > 0.0
        if self.coated and core_radii is None:
            raise ValueError("the coating model needs the core radius of every element")
        self.mesh = DeviceMesh(coords, conn, radii, layer, device=self.device, mu=mu_elem,
                               core_radii=core_radii if self.coated else None)
        self.beam = DeviceBeam(self.mesh, section, v_ref=v_ref)
        self.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        self.cp = L.ContactParams(k_pen, k_t_ratio, mu, smoothing_delta, g_on, g_off, int(allow_deactivation),
                                  float(co.get("stiffness", 0.0)), float(co.get("damping", 0.0)),
                                  float(co.get("mu", 0.0)), float(co.get("k_t_ratio", 0.5)), float(co.get("dt", 0.0)))
        self.bp = L.BPParams(margin, int(exclude_shared), int(exclude_same_layer and layer is not None),
                             int(midpoint_prescreening), prescreening_margin)
        dev = self.device
        nd = self.mesh.ndof
        self.pairs = DevicePairTable(dev, coating=self.coated)
        self._spare = DevicePairTable(dev, coating=self.coated)
        self.pattern = DeviceContactPattern(self.mesh)
        self.f_int = torch.zeros(nd, dtype=torch.float64, device=dev)
        self.R = torch.zeros(nd, dtype=torch.float64, device=dev)
        self.norm2 = torch.zeros(1, dtype=torch.float64, device=dev)
        self.cands = torch.zeros(2 * 1024, dtype=torch.int32, device=dev)
        # mixed fast path: float node / element records and the float copy of the pair state
        self.node32 = torch.zeros(L.NODE32_STRIDE * max(self.mesh.n_nodes, 1), dtype=torch.float32, device=dev)
        self.elem32 = torch.zeros(L.ELEM32_STRIDE * max(self.mesh.n_elems, 1), dtype=torch.float32, device=dev)
        self.pairs32 = DevicePairTable32(dev, per_slot_mu=mu_elem is not None, coating=self.coated)
        self._state_in32 = False
        self.update_reference_frames()
        self._alloc_outputs()
        self.stats: dict = {}
        self.graph = None
        self.gather_variant = L.XK_GATHER_DEFAULT
        self.autotune = True
        self.tune_launch_shapes = False  # also tune the launch shapes in capture (tune(shapes=True))
        self.tune_shapes = {}
        self._pair_block = 0  # 0: the kernels' default CTA size
        self._tuned_for = None
        # learned candidate pruning (``set_pruner``); the exact path verifies it every ``verify_every`` detections
        self.pruner = None
        self.verify_every = 10
        # mixed engine: detection narrowphase in float with the exact routine for the pairs near the
        # active-set thresholds (xk_narrowphase_screened); the active set is the exact one either way
        self.screened_detection = True
        self._n_exact = torch.zeros(1, dtype=torch.int32, device=self.device)
        self._n_detect = 0
        self.prune_stats = {"detections": 0, "verified": 0, "candidates": 0, "kept": 0, "missed": 0}
        self._verify_tables = None  # scratch pair tables of the pruner's verification, kept across detections
        # with trace_phases, detect records a CUDA event after each phase (no extra synchronisation);
        # phase_ms() reads the times of the last detection
        self.trace_phases = False
        self._phase_marks: list = []

    # ------------------------------------------------------------------ buffers
    @property
    def t_dtype(self):
        return torch.float64 if self.precision == L.XK_FP64 else torch.float32

    def _alloc_outputs(self):
        dev = self.device
        self.K_beam = torch.zeros(36 * max(self.beam.nnzb, 1), dtype=self.t_dtype, device=dev)
        self.rec = torch.zeros(L.REC_STRIDE[L.XK_OUT_COMBINED] * self.pattern.cap_members, dtype=self.t_dtype,
                               device=dev)
        self.K_c = torch.zeros(9 * max(self.pattern.cap_blocks, 1), dtype=self.t_dtype, device=dev)
        self.graph = None

    def update_reference_frames(self, stream=None):
        """Recompute per-element reference data after the reference coordinates changed."""
        self.beam.update_reference_frames(stream)
        L.call("xk_beam_prepare32", C.byref(self.mesh.c), ptr(self.beam.elem_ref), ptr(self.elem32),
               stream_handle(stream))

    def _to32(self, s):
        self.pairs32.ensure(self.pairs.cap)
        L.call("xk_pairs_to32", C.byref(self.mesh.c), C.byref(self.pairs.c), C.byref(self.pattern.c),
               C.byref(self.pairs32.c), s)
        self._state_in32 = True

    def sync_state(self, stream=None):
        """Bring the double pair table up to date with the float copy (mixed path)."""
        if self._state_in32:
            L.call("xk_pairs_from32", C.byref(self.pairs32.c), C.byref(self.pairs.c), stream_handle(stream))
            self._state_in32 = False

    def set_precision(self, precision):
        p = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        if p != self.precision:
            self.precision = p
            self._alloc_outputs()

    # ------------------------------------------------------------------ per increment
    def candidates(self, u: torch.Tensor, stream=None):
        """Broadphase + filters at X + u: (candidate rows int32 [2n] on the device, n)."""
        s = stream_handle(stream)
        n_out, n_raw, n_pre = C.c_int64(0), C.c_int64(0), C.c_int64(0)
        for _ in range(3):
            code = L.call("xk_broadphase", C.byref(self.mesh.c), ptr(u), C.byref(self.bp), ptr(self.cands),
                          self.cands.numel() // 2, C.byref(n_out), C.byref(n_raw), C.byref(n_pre), s,
                          allow=(L.XK_ERR_CAPACITY,))
            if code == L.XK_OK:
                break
            self.cands = torch.zeros(2 * int(n_out.value * 1.25 + 1024), dtype=torch.int32, device=self.device)
        self._bp_counts = (int(n_raw.value), int(n_pre.value))
        return self.cands, int(n_out.value)

    def set_coating_dt(self, dt: float):
        """The step's pseudo-time increment of the coating dashpot (``load_frac - load_frac_prev`` in the
        reference's Newton loop, ``_newton_steps.py:112``); a captured graph is recorded again."""
        self.cp.coat_dt = float(dt)
        self.graph = None

    def end_step(self, stream=None):
        """At a converged step: coating_compression_prev <- coating_compression for every pair
        (``contact/solver/process.py:539-545``)."""
        if not self.coated:
            return
        if self._state_in32:
            t = self.pairs32.t
            t["coat_cc_prev"].copy_(t["coat_cc"])
        else:
            n = self.pairs.n
            self.pairs.t["coat_cc_prev"][:n].copy_(self.pairs.t["coat_cc"][:n])

    def set_pruner(self, pruner, verify_every: int = 10):
        """Use a trained ``PairPruner`` at detection; every ``verify_every``-th detection checks it exactly."""
        if self.coated:
            raise NotImplementedError("candidate pruning is not combined with the coating model")
        self.pruner = pruner
        self.verify_every = max(1, int(verify_every))

    def _prune(self, u, cands, nc, s, stream):
        """Candidates the pruner keeps (plus every pair with history), verified exactly when due."""
        pr = self.pruner
        feat, hist = pr.features(self.mesh, self.node32, cands, nc, self.pairs, stream)
        self._mark("prune_features", stream)
        logit = pr.logits(feat, nc, stream)
        self._mark("prune_scores", stream)
        kept = torch.empty(2 * max(nc, 1), dtype=torch.int32, device=self.device)
        nk, failed = C.c_int64(0), C.c_int32(0)
        err = ptr(pr._tc_err) if pr.backend == "tcgen05" else None
        # one synchronisation: the kept count and the scoring's error word come back together; after an
        # expired tensor-core wait the scores are undefined and the select keeps every candidate
        L.call("xk_prune_select", ptr(cands), nc, ptr(logit), ptr(hist), pr.threshold, 0, err, ptr(kept),
               C.byref(nk), C.byref(failed), s)
        self._mark("prune_select", stream)
        nk = int(nk.value)
        st = self.prune_stats
        st["detections"] += 1
        st["candidates"] += nc
        if failed.value:
            st["scoring_failed"] = st.get("scoring_failed", 0) + 1
            st["kept"] += nc
            return cands, nc
        if self._n_detect % self.verify_every == 0:
            # verification: the active-set narrowphase of every pruned candidate (the screened one in the
            # mixed engine, whose active sets are the exact path's); any that would turn ACTIVE is a missed
            # contact and the whole candidate set is used instead
            st["verified"] += 1
            dropped = torch.empty(2 * max(nc - nk, 1), dtype=torch.int32, device=self.device)
            nd = C.c_int64(0)
            L.call("xk_prune_select", ptr(cands), nc, ptr(logit), ptr(hist), pr.threshold, 1, None, ptr(dropped),
                   C.byref(nd), None, s)
            nd = int(nd.value)
            missed = 0
            if nd:
                if self._verify_tables is None:
                    self._verify_tables = (DevicePairTable(self.device, cap=16), DevicePairTable(self.device, cap=16))
                empty, tmp = self._verify_tables
                empty.set_n(0)
                tmp.reserve(nd + 16, keep=False)
                L.call("xk_pairs_merge", C.byref(self.mesh.c), C.byref(empty.c), ptr(dropped), nd, C.byref(tmp.c), s)
                tmp.set_n(tmp.c.n)
                if self.precision == L.XK_MIXED and self.screened_detection:
                    L.call("xk_narrowphase_screened", C.byref(self.mesh.c), C.byref(tmp.c), ptr(u), ptr(self.node32),
                           C.byref(self.cp), ptr(self._n_exact), s)
                else:
                    L.call("xk_narrowphase", C.byref(self.mesh.c), C.byref(tmp.c), ptr(u), C.byref(self.cp), 1, s)
                missed = int((tmp.t["status"][: tmp.n] != 0).sum().item())
            st["missed"] += missed
            st["last_verify_missed"] = missed
            if missed:
                st["kept"] += nc
                return cands, nc
        st["kept"] += nk
        self._merge_pruned = True  # the merge drops the pristine old pairs that are not kept
        return kept, nk

    def _mark(self, name: str, stream=None):
        if self.trace_phases:
            e = torch.cuda.Event(enable_timing=True)
            e.record(stream if stream is not None else torch.cuda.current_stream())
            self._phase_marks.append((name, e))

    def phase_ms(self) -> dict:
        """GPU-timeline time (ms) of each phase of the last detection, when ``trace_phases`` is set: the
        span between the events recorded at the ends of consecutive phases."""
        m = self._phase_marks
        if len(m) < 2:
            return {}
        m[-1][1].synchronize()
        return {name: m[k - 1][1].elapsed_time(e) for k, (name, e) in enumerate(m) if k > 0}

    def detect(self, u: torch.Tensor, stream=None) -> dict:
        """Broadphase, pair-table merge, active-set narrowphase and contact pattern at X + u."""
        s = stream_handle(stream)
        self._phase_marks = []
        self._mark("start", stream)
        self.sync_state(stream)
        self._mark("table_back", stream)
        cands, nc = self.candidates(u, stream)
        self._mark("broadphase", stream)
        n_raw, n_pre = self._bp_counts
        n_all = nc
        self._merge_pruned = False
        screened = self.precision == L.XK_MIXED and self.screened_detection and not self.coated
        if self.pruner is not None or screened:  # node records at u: pruning features, screened narrowphase
            L.call("xk_nodes_prepare", C.byref(self.mesh.c), ptr(u), ptr(u), ptr(self.node32), s)
        if self.pruner is not None:
            cands, nc = self._prune(u, cands, nc, s, stream)
            self._mark("prune_verify", stream)
        self._n_detect += 1
        need = self.pairs.n + nc
        if self._spare.cap < need:
            self._spare.reserve(int(need * 1.25) + 64, keep=False)
        L.call("xk_pairs_merge_pruned" if self._merge_pruned else "xk_pairs_merge", C.byref(self.mesh.c),
               C.byref(self.pairs.c), ptr(cands), nc, C.byref(self._spare.c), s)
        self._spare.set_n(self._spare.c.n)
        self.pairs, self._spare = self._spare, self.pairs
        self._mark("merge", stream)
        if screened:
            L.call("xk_narrowphase_screened", C.byref(self.mesh.c), C.byref(self.pairs.c), ptr(u), ptr(self.node32),
                   C.byref(self.cp), ptr(self._n_exact), s)
        else:
            L.call("xk_narrowphase", C.byref(self.mesh.c), C.byref(self.pairs.c), ptr(u), C.byref(self.cp), 1, s)
        self._mark("narrowphase", stream)
        self.pattern.build(self.pairs, stream)
        self._mark("pattern", stream)
        # read while the stream is idle after the pattern build, before the float copy is queued, so that
        # detect returns without waiting for it
        n_exact = int(self._n_exact.item()) if screened else self.pairs.n
        if self.precision == L.XK_MIXED:
            self._to32(s)
            self._mark("float_table", stream)
        if (self.rec.numel() != L.REC_STRIDE[L.XK_OUT_COMBINED] * self.pattern.cap_members
                or self.K_c.numel() < 9 * self.pattern.cap_blocks):
            self._alloc_outputs()
        self.graph = None
        self.stats = {"raw": n_raw, "prefilter": n_pre, "candidates": n_all, "kept_candidates": nc,
                      "pairs": self.pairs.n, "members": self.pattern.n_members, "contact_blocks": self.pattern.nnzb,
                      "contact_blocks_full": self.pattern.nnzb_full,
                      "narrowphase_exact": n_exact}
        return self.stats

    # ------------------------------------------------------------------ per iteration
    def assemble(self, u: torch.Tensor, u_ref: torch.Tensor | None = None, f_ext: torch.Tensor | None = None,
                 fixed: torch.Tensor | None = None, stream=None, *, tangent: bool = True):
        """One Newton iteration's assembly: R (with its squared norm), K_beam and K_c.

        The independent parts run on separate streams and join before the
        residual (in a captured graph they become parallel branches): the other
        pairs' narrowphase, the beam elements, and the member kernel followed by
        the contact tangent; the force gather waits for the members and the beam.
        Every kernel writes its own outputs, so the results do not depend on the
        overlap.
        """
        main = stream if stream is not None else torch.cuda.current_stream()
        s = stream_handle(main)
        p = self.precision
        pat = C.byref(self.pattern.c)
        so, sb, st = self._side_streams()
        if p == L.XK_MIXED:
            if not self._state_in32:
                self._to32(s)
            self.pairs32.c.block = self._pair_block  # the float table's struct is rebuilt when it grows
            L.call("xk_nodes_prepare", C.byref(self.mesh.c), ptr(u), ptr(u_ref), ptr(self.node32), s)
        so.wait_stream(main)
        sb.wait_stream(main)
        # other pairs' narrowphase
        if p == L.XK_MIXED:
            L.call("xk_pair_step32", C.byref(self.pairs32.c), ptr(self.node32), C.byref(self.cp), ptr(self.rec),
                   L.XK_PAIRS_OTHERS, stream_handle(so))
        else:
            L.call("xk_pair_step", C.byref(self.mesh.c), C.byref(self.pairs.c), pat, ptr(u), ptr(u_ref),
                   C.byref(self.cp), L.XK_STAGE_NARROW | L.XK_STAGE_NO_MEMBERS, p, L.XK_OUT_COMBINED,
                   ptr(self.rec), stream_handle(so))
        # beam elements
        if p == L.XK_MIXED:
            L.call("xk_beam_assemble32", C.byref(self.mesh.c), C.byref(self.beam.section), ptr(self.elem32),
                   C.byref(self.beam.plan), ptr(self.node32), ptr(self.f_int), ptr(self.K_beam) if tangent else None,
                   stream_handle(sb))
        else:
            self.beam.assemble(u, p, self.f_int, self.K_beam if tangent else None, sb)
        # contributing pairs, then the contact tangent from their records
        if p == L.XK_MIXED:
            L.call("xk_pair_step32", C.byref(self.pairs32.c), ptr(self.node32), C.byref(self.cp), ptr(self.rec),
                   L.XK_PAIRS_MEMBERS, s)
        else:
            L.call("xk_pair_step", C.byref(self.mesh.c), C.byref(self.pairs.c), pat, ptr(u), ptr(u_ref),
                   C.byref(self.cp), L.XK_STAGE_ALL | L.XK_STAGE_NO_OTHERS, p, L.XK_OUT_COMBINED, ptr(self.rec), s)
        gather = tangent and self.pattern.nnzb > 0
        # the element-side schedules leave per-element force sums that the residual reads
        elem_force = gather and self.gather_variant == L.XK_GATHER_SIDES
        sums_done = None
        if gather:
            st.wait_stream(main)
            if elem_force:  # element sums, then the blocks; the residual needs only the sums
                L.call("xk_contact_gather_tangent", pat, ptr(self.rec), p, L.XK_OUT_COMBINED, L.XK_WHICH_COMBINED,
                       L.XK_GATHER_SIDES_SUMS, ptr(self.K_c), stream_handle(st))
                sums_done = torch.cuda.Event()
                sums_done.record(st)
                L.call("xk_contact_gather_tangent", pat, ptr(self.rec), p, L.XK_OUT_COMBINED, L.XK_WHICH_COMBINED,
                       L.XK_GATHER_SIDES_BLOCKS, ptr(self.K_c), stream_handle(st))
            else:
                L.call("xk_contact_gather_tangent", pat, ptr(self.rec), p, L.XK_OUT_COMBINED, L.XK_WHICH_COMBINED,
                       self.gather_variant, ptr(self.K_c), stream_handle(st))
        # residual after the members (or the tangent gather's element sums) and the beam
        main.wait_stream(sb)
        if elem_force:
            main.wait_event(sums_done)
            L.call("xk_contact_gather_force_elem", pat, p, ptr(self.f_int), -1.0, ptr(f_ext), ptr(fixed),
                   ptr(self.R), ptr(self.norm2), s)
        else:
            L.call("xk_contact_gather_force", pat, ptr(self.rec), p, L.XK_OUT_COMBINED, L.XK_WHICH_COMBINED,
                   ptr(self.f_int), -1.0, ptr(f_ext), ptr(fixed), ptr(self.R), ptr(self.norm2), s)
        main.wait_stream(so)
        if gather:
            main.wait_stream(st)
        return self.R

    def _side_streams(self):
        if getattr(self, "_streams", None) is None:
            self._streams = tuple(torch.cuda.Stream(device=self.device) for _ in range(3))
        return self._streams

    def pair_step(self, u: torch.Tensor, u_ref: torch.Tensor | None = None, stream=None):
        """The pair part of ``assemble``: narrowphase of every pair and the member records."""
        s = stream_handle(stream)
        pat = C.byref(self.pattern.c)
        if self.precision == L.XK_MIXED:
            if not self._state_in32:
                self._to32(s)
            L.call("xk_nodes_prepare", C.byref(self.mesh.c), ptr(u), ptr(u_ref), ptr(self.node32), s)
            L.call("xk_pair_step32", C.byref(self.pairs32.c), ptr(self.node32), C.byref(self.cp), ptr(self.rec),
                   L.XK_PAIRS_ALL, s)
        else:
            L.call("xk_pair_step", C.byref(self.mesh.c), C.byref(self.pairs.c), pat, ptr(u), ptr(u_ref),
                   C.byref(self.cp), L.XK_STAGE_ALL, self.precision, L.XK_OUT_COMBINED, ptr(self.rec), s)

    def _time_calls(self, fn, reps: int) -> float:
        s = torch.cuda.current_stream()
        for _ in range(2):
            fn(s)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        for _ in range(reps):
            fn(s)
        b.record(s)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    def tune(self, reps: int = 5, shapes: bool = False) -> dict:
        """Time the contact-tangent reduction schedules on the current records and keep the fastest;
        with ``shapes`` also the launch shapes: the CTA size of the float pair kernels and the persistent
        CTAs per SM of the element-side block gather.

        Run after an ``assemble`` of the increment (the records must be current);
        values do not depend on the choice beyond rounding order (the schedules) or at all (the shapes).
        """
        times = {}
        if self.pattern.nnzb == 0:
            return times
        pc = C.byref(self.pattern.c)
        variants = [L.XK_GATHER_LANES, L.XK_GATHER_CHUNKS]
        if self.pattern.c.sides_ok == 1:  # every block fits four inline terms (wire meshes)
            variants.append(L.XK_GATHER_SIDES)
        for v in variants:
            times[v] = self._time_calls(lambda s, v=v: L.call(
                "xk_contact_gather_tangent", pc, ptr(self.rec), self.precision, L.XK_OUT_COMBINED,
                L.XK_WHICH_COMBINED, v, ptr(self.K_c), stream_handle(s)), reps)
        self.gather_variant = min(times, key=times.get)
        self.tune_times = times
        self._tuned_for = (self.pattern.version, self.precision)
        if shapes:
            self.tune_shapes = self._tune_shapes(reps)
        return times

    def _tune_shapes(self, reps: int) -> dict:
        """Launch shapes, each timed alone on the current state; the defaults are among the candidates."""
        out = {}
        if self.precision == L.XK_MIXED and self._state_in32:
            q = self.pairs32.c
            t = {}
            for bs in (128, 256):
                q.block = bs
                t[bs] = self._time_calls(lambda s: L.call("xk_pair_step32", C.byref(q), ptr(self.node32),
                                                          C.byref(self.cp), ptr(self.rec), L.XK_PAIRS_ALL,
                                                          stream_handle(s)), reps)
            q.block = min(t, key=t.get)
            self._pair_block = q.block
            out["pair_block"] = {"times_ms": t, "chosen": q.block, "default": 256}
        if self.gather_variant == L.XK_GATHER_SIDES:
            pat = self.pattern.c
            t = {}
            for per_sm in (4, 8, 12, 16, 24):
                pat.sides_per_sm = per_sm
                t[per_sm] = self._time_calls(lambda s: L.call(
                    "xk_contact_gather_tangent", C.byref(pat), ptr(self.rec), self.precision, L.XK_OUT_COMBINED,
                    L.XK_WHICH_COMBINED, L.XK_GATHER_SIDES_BLOCKS, ptr(self.K_c), stream_handle(s)), reps)
            pat.sides_per_sm = min(t, key=t.get)
            out["sides_ctas_per_sm"] = {"times_ms": t, "chosen": pat.sides_per_sm,
                                        "default": 16 if self.precision == L.XK_MIXED else 8}
        self.graph = None
        return out

    def capture(self, u, u_ref=None, f_ext=None, fixed=None):
        """Record ``assemble`` on these (static) buffers as a CUDA graph."""
        st = torch.cuda.Stream(device=self.device)
        st.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(st):
            self.assemble(u, u_ref, f_ext, fixed, stream=st)  # warm-up outside capture
        torch.cuda.current_stream().wait_stream(st)
        if self.autotune and self._tuned_for != (self.pattern.version, self.precision):
            torch.cuda.synchronize()
            self.tune(shapes=self.tune_launch_shapes)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=st):
            self.assemble(u, u_ref, f_ext, fixed, stream=st)
        self.graph = g
        return g

    def replay(self):
        self.graph.replay()

    # ------------------------------------------------------------------ host views
    def pair_state(self) -> dict:
        """Host copy of the pair table (after syncing the float copy in mixed mode)."""
        self.sync_state()
        return self.pairs.to_host()

    def residual_norm(self) -> float:
        return float(np.sqrt(self.norm2.item()))

    def K_beam_csr(self, vals: torch.Tensor | None = None) -> sp.csr_matrix:
        """The full beam tangent from its stored (row <= column) blocks and their transposes; ``vals``
        (e.g. a ``HostPipeline`` result) instead of the engine's own values."""
        return self.beam.to_csr(self.K_beam if vals is None else vals)

    def K_contact_csr(self, vals: torch.Tensor | None = None) -> sp.csr_matrix:
        """The full contact tangent from its stored (row <= column) blocks and their mirrors."""
        return self.pattern.to_csr(self.K_c if vals is None else vals, self.mesh.ndof)

    def K_total_csr(self) -> sp.csr_matrix:
        return (self.K_beam_csr() + self.K_contact_csr()).tocsr()


class HostPipeline:
    """Newton-iteration assembly from host inputs to host outputs, copies overlapped with compute.

    ``submit(u, u_ref)`` copies the pinned host inputs into the engine's graph
    inputs, replays the captured assembly, snapshots R, K_beam and K_c into one
    of two device staging sets and starts their copy to pinned host memory on a
    copy stream; ``result(ticket)`` waits for that copy and returns the host
    arrays.  The read-back of one step runs while the next step is copied in
    and assembled.  The two staging sets and two host sets are reused in turn,
    so a ticket's arrays stay valid until two more steps have been submitted.

    With ``read_tangent=False`` only R and its squared norm come back (a caller
    whose linear solve runs on the device, from the engine's K_beam and K_c,
    needs nothing else on the host): ``result`` returns (R, None, None) and
    ``residual_norm2(ticket)`` the norm.
    """

    def __init__(self, engine: AssemblyEngine, read_tangent: bool = True):
        self.eng = engine
        self.read_tangent = bool(read_tangent)
        dev = engine.device
        nd = engine.mesh.ndof
        self.u_in = torch.zeros(nd, dtype=torch.float64, device=dev)
        self.ur_in = torch.zeros(nd, dtype=torch.float64, device=dev)
        self.nkc = 9 * engine.pattern.nnzb if self.read_tangent else 0
        kd = engine.K_beam.dtype
        nkb = engine.K_beam.numel() if self.read_tangent else 1
        # R with its squared norm appended (nd + 1 doubles), K_beam, K_c
        self.dev_out = [(torch.empty(nd + 1, dtype=torch.float64, device=dev),
                         torch.empty(nkb, dtype=kd, device=dev),
                         torch.empty(max(self.nkc, 1), dtype=engine.K_c.dtype, device=dev)) for _ in range(2)]
        self.host_out = [tuple(torch.empty(t.numel(), dtype=t.dtype).pin_memory() for t in d) for d in self.dev_out]
        self.copy_in = torch.cuda.Stream(device=dev)
        self.copy_out = torch.cuda.Stream(device=dev)
        self._slot_free = [None, None]  # events: the staging / host set may be overwritten
        self._inputs_free = None  # event: the replay has read the inputs
        self._done = {}
        self._last = 0
        self.n = 0
        engine.capture(self.u_in, self.ur_in)

    def submit(self, u_host: torch.Tensor, u_ref_host: torch.Tensor) -> int:
        eng, main = self.eng, torch.cuda.current_stream()
        k = self.n % 2
        if self._inputs_free is not None:
            self.copy_in.wait_event(self._inputs_free)
        with torch.cuda.stream(self.copy_in):
            self.u_in.copy_(u_host, non_blocking=True)
            self.ur_in.copy_(u_ref_host, non_blocking=True)
        main.wait_stream(self.copy_in)
        eng.replay()
        self._inputs_free = torch.cuda.Event()
        self._inputs_free.record(main)
        if self._slot_free[k] is not None:
            main.wait_event(self._slot_free[k])
        R, Kb, Kc = self.dev_out[k]
        nd = eng.R.numel()
        R[:nd].copy_(eng.R, non_blocking=True)
        R[nd:].copy_(eng.norm2, non_blocking=True)
        if self.read_tangent:
            Kb.copy_(eng.K_beam, non_blocking=True)
        if self.nkc:
            Kc[: self.nkc].copy_(eng.K_c[: self.nkc], non_blocking=True)
        self.copy_out.wait_stream(main)
        hR, hKb, hKc = self.host_out[k]
        with torch.cuda.stream(self.copy_out):
            hR.copy_(R, non_blocking=True)
            if self.read_tangent:
                hKb.copy_(Kb, non_blocking=True)
            if self.nkc:
                hKc[: self.nkc].copy_(Kc[: self.nkc], non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(self.copy_out)
        self._slot_free[k] = ev
        self._done[self.n] = (ev, k)
        self.n += 1
        return self.n - 1

    def result(self, ticket: int):
        """(R, K_beam values, K_c values) of a submitted step as pinned host tensors ((R, None, None) without
        the tangent read-back)."""
        ev, k = self._done.pop(ticket)
        ev.synchronize()
        self._last = k
        hR, hKb, hKc = self.host_out[k]
        nd = self.u_in.numel()
        if not self.read_tangent:
            return hR[:nd], None, None
        return hR[:nd], hKb, hKc[: self.nkc]

    def residual_norm2(self) -> float:
        """The squared residual norm of the step whose ``result`` was taken last (FP64, fixed order)."""
        return float(self.host_out[self._last][0][self.u_in.numel()])

    @property
    def bytes_in(self) -> int:
        return 2 * self.u_in.numel() * 8

    @property
    def bytes_out(self) -> int:
        r = self.dev_out[0][0].numel() * 8
        if not self.read_tangent:
            return r
        return r + self.dev_out[0][1].numel() * self.dev_out[0][1].element_size() + self.nkc * self.dev_out[0][2].element_size()
