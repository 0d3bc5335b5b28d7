"""Benchmark: assembly + contact evaluations per second of one Newton iteration.

Workload: the 1027-wire hexagonally layered strand (18 layers, wire diameter
0.5 mm, lay pitch 20 mm, 4 pitches, 24 elements per pitch: 99,619 nodes,
98,592 CR beam elements), nodes perturbed by seeded Gaussian noise, contact
forced by a nominal layer gap of -0.005 d; synthetic inputs of the reference's
shapes.  One step is one Newton-iteration assembly on the device: the fused
pair kernel over every pair of the table (frozen narrowphase, Huber normal
force, Coulomb return mapping, pair tangent), the CR beam f_int and K_T, the
residual with its FP64 norm and the contact tangent K_c.  The per-increment
detection (broadphase, merge, active set, pattern) runs before the timed
region and is reported separately.

metric value = (N_e + N_c) / seconds per step, N_c = pairs in the table.
The headline is the mixed-precision path; the plain FP64 path is timed in the
same run (``fp64_plain``) together with the error of mixed against FP64.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for _p in (str(ROOT), str(ROOT / "xkep-cae_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "assembly+contact evals/s at 1027-wire vs FP64 plain on GB300; err vs FP64"
UNIT = "evals/s"


# --------------------------------------------------------------------------- helpers


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        out_dir = Path(os.environ.get("XK_CLOCKS_DIR", tempfile.gettempdir()))
        self.path = out_dir / f"clocks_{os.getpid()}.csv"
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self) -> dict:
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def slab_elems(nel: int, frac: float) -> int:
    return max(2, int(round(nel * frac)))


def slab_workload(w, frac: float, index: int = 0):
    """Slab ``index`` of every wire, ``frac`` of its length each (slab 0 is the first ``frac``): a
    bounded sample of the same strand for CPU timing."""
    from xkgpu import strand as S

    st = w.strand
    nel = st.n_elems_per_wire
    keep_el = slab_elems(nel, frac)
    e0 = index * keep_el
    if e0 + keep_el > nel:
        raise ValueError(f"slab {index} of {keep_el} elements does not fit a wire of {nel}")
    npw = nel + 1
    nodes, elems = [], []
    for wi in range(len(st.wires)):
        nodes.append(np.arange(wi * npw + e0, wi * npw + e0 + keep_el + 1))
        elems.append(np.arange(wi * nel + e0, wi * nel + e0 + keep_el))
    nodes = np.concatenate(nodes)
    elems = np.concatenate(elems)
    remap = -np.ones(st.n_nodes, dtype=np.int64)
    remap[nodes] = np.arange(nodes.size)
    sub = S.Strand(coords=st.coords[nodes], conn=remap[st.conn[elems]].astype(np.int32),
                   elem_layer=st.elem_layer[elems], radii=st.radii[elems], wires=st.wires,
                   wire_diameter=st.wire_diameter, pitch=st.pitch, length=st.length, n_elems_per_wire=keep_el)
    u = w.u.reshape(-1, 6)[nodes].ravel().copy()
    return sub, u


def oracle_sample_timing(w, frac: float, reps: int = 1, prepared=None, index: int = 0):
    """Time the oracle (NumPy port) on a slab of the strand; returns (units, seconds, prepared)."""
    from oracle import beam as ob
    from oracle import contact as oc

    if prepared is None:
        sub, u = slab_workload(w, frac, index)
        cd = oc.deformed_coords(sub.coords, u)
        table, _, _ = oc.detect(oc.empty_table(), cd, sub.conn, sub.radii, elem_layer=sub.elem_layer,
                                exclude_same_layer=True)
        table = oc.update_geometry(table, cd)
        prepared = (sub, u, table)
    sub, u, table = prepared
    sec = ob.Section(**w.section, scf=None)
    u1 = u * 1.001
    t0 = time.perf_counter()
    for _ in range(reps):
        oc.contact_iteration(table, sub.coords, u1, u, sub.ndof, k_pen=w.k_pen, k_t_ratio=w.k_t_ratio, mu_eff=w.mu)
        ob.assemble_beam(sub.coords, sub.conn, u1, sec)
    dt = time.perf_counter() - t0
    units = reps * (sub.n_elems + table["ea"].shape[0])
    return units, dt, prepared


def pair_kernel_bytes(n_nodes, n_elems, n_others, n_members, mixed: bool):
    """Algorithmic (compulsory) DRAM bytes of one pair step.

    FP64 path (double state): node data X, u, u_ref once per node (72 B),
    conn and radius once per element (16 B); a non-contributing pair reads its
    list entry, keys and previous frame (60 B) and writes s, t, gap and the
    frame (96 B); a contributing pair reads node ids, keys, status and friction
    state (126 B), writes the updated state (138 B) and its 16-double record.

    Mixed path (float state): the node-preparation kernel reads X, u, u_ref
    (72 B) and writes a 64 B node record that the pair kernels read back
    (64 B); element radii 8 B; a non-contributing pair reads 48 B (node ids,
    radius sum, previous normal and t1) and writes 36 B (s, t, gap, normal,
    t1); a contributing pair reads 78 B, writes 70 B and its 64 B record.
    """
    if mixed:
        return (72 + 64 + 64) * n_nodes + 8 * n_elems + 84 * n_others + 212 * n_members
    return 72 * n_nodes + 16 * n_elems + 156 * n_others + n_members * (264 + 128)


def gather_tangent_bytes(n_members, n_contrib, nnzb, mixed: bool, sides: bool = False, n_elems: int = 0):
    """Algorithmic DRAM bytes of one contact-tangent gather (all its launches).

    Each contributing pair's record is read once (16 values: 64 B float, 128 B
    double) and each stored 3x3 block (row <= column; the block at the mirrored
    position has the same values and is not written) once (36 B float, 72 B
    double); re-reads
    of a record by the blocks it feeds are L2 traffic.  Contributor-list
    schedules also read each list entry (4 B) and block pointer (4 B).  The
    element-side schedule instead reads each member's two element-incidence
    entries (8 B) and the element pointers (4 B), writes every element's three
    tangent sums (12 values each: the 9 of the sum and the weight slots that a
    term load reads) and its 8 force-sum values, reads the tangent sums back
    once, and reads four inline terms per block (16 B).
    """
    w = 4 if mixed else 8
    if sides:
        return (16 * w * n_members + 8 * n_members + 4 * (n_elems + 1) + (36 + 8 + 36) * w * n_elems
                + 16 * nnzb + 9 * w * nnzb)
    return 16 * w * n_members + 4 * n_contrib + 4 * (nnzb + 1) + 9 * w * nnzb


def kernel_roofline_mixed(eng, u1, u0, peak, reps: int = 50) -> list:
    """Every launch of the mixed assembly alone: CUDA-event time (mean over ``reps`` back-to-back calls
    captured in one CUDA graph and replayed, so that host launch overhead does not pace the small
    kernels; ``us_eager`` is the same loop launched from Python), algorithmic bytes and the fraction of
    the HBM peak.

    Algorithmic bytes (compulsory traffic, each array read or written once):
    node preparation 72 B read (X, u, u_ref) + 64 B record written per node; other pairs 48 B read
    + 36 B written per pair + the 64 B node records; the beam 64 B element record + 432 B of its three
    stored 6x6 float blocks per element, the node records and the 48 B double f_int rows per node;
    contributing pairs 78 B read + 70 B written + a 64 B record each + the node records; the element
    sums 64 B record + 8 B incidence per member, 4 B pointer and 80 floats written per element; the
    block gather 16 B of inline term codes and 36 B written per stored block, 36 floats of element
    sums read per element; the residual 48 B f_int read, 48 B R written and 2 x 32 B element force
    sums per node.
    """
    import ctypes as C

    import torch

    from xkgpu import _lib as L
    from xkgpu.device import ptr, stream_handle

    s = torch.cuda.current_stream()
    pat = eng.pattern
    n_n, n_e = eng.mesh.n_nodes, eng.mesh.n_elems
    n_m = pat.n_members
    n_o = eng.pairs.n - n_m
    nb = pat.nnzb
    pc = C.byref(pat.c)
    eng.assemble(u1, u0)  # records and element sums current
    launches = [
        ("k_nodes_prepare", lambda sh: L.call("xk_nodes_prepare", C.byref(eng.mesh.c), ptr(u1), ptr(u0), ptr(eng.node32),
                                              sh), 136 * n_n),
        ("k_pair_other32 (+ near-parallel)", lambda sh: L.call("xk_pair_step32", C.byref(eng.pairs32.c),
                                                               ptr(eng.node32), C.byref(eng.cp), ptr(eng.rec),
                                                               L.XK_PAIRS_OTHERS, sh), 84 * n_o + 64 * n_n),
        ("k_beam32e (ordered wires, one launch)", lambda sh: L.call("xk_beam_assemble32", C.byref(eng.mesh.c),
                                                        C.byref(eng.beam.section), ptr(eng.elem32),
                                                        C.byref(eng.beam.plan), ptr(eng.node32), ptr(eng.f_int),
                                                        ptr(eng.K_beam), sh), (64 + 432) * n_e + (64 + 48) * n_n),
        ("k_pair_member32 (+ near-parallel)", lambda sh: L.call("xk_pair_step32", C.byref(eng.pairs32.c),
                                                                ptr(eng.node32), C.byref(eng.cp), ptr(eng.rec),
                                                                L.XK_PAIRS_MEMBERS, sh), 212 * n_m + 64 * n_n),
        ("k_elem_sums_rec", lambda sh: L.call("xk_contact_gather_tangent", pc, ptr(eng.rec), eng.precision,
                                              L.XK_OUT_COMBINED, L.XK_WHICH_COMBINED, L.XK_GATHER_SIDES_SUMS,
                                              ptr(eng.K_c), sh), 72 * n_m + 4 * (n_e + 1) + 320 * n_e),
        ("k_gather_tangent_sides", lambda sh: L.call("xk_contact_gather_tangent", pc, ptr(eng.rec), eng.precision,
                                                     L.XK_OUT_COMBINED, L.XK_WHICH_COMBINED, L.XK_GATHER_SIDES_BLOCKS,
                                                     ptr(eng.K_c), sh), (16 + 36) * nb + 144 * n_e),
        ("k_gather_force_elem", lambda sh: L.call("xk_contact_gather_force_elem", pc, eng.precision, ptr(eng.f_int), -1.0,
                                                  None, None, ptr(eng.R), ptr(eng.norm2), sh), (48 + 48 + 64) * n_n),
    ]
    out = []
    cs = torch.cuda.Stream()
    for name, fn, nbytes in launches:
        sh = stream_handle(s)
        for _ in range(3):
            fn(sh)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        for _ in range(reps):
            fn(sh)
        b.record(s)
        torch.cuda.synchronize()
        t_eager = a.elapsed_time(b) / 1e3 / reps
        g = torch.cuda.CUDAGraph()
        cs.wait_stream(s)
        with torch.cuda.graph(g, stream=cs):
            h = stream_handle(cs)
            for _ in range(reps):
                fn(h)
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        a.record(s)
        g.replay()
        b.record(s)
        torch.cuda.synchronize()
        t = a.elapsed_time(b) / 1e3 / reps
        del g
        out.append({"kernel": name, "us": round(1e6 * t, 2), "us_eager": round(1e6 * t_eager, 2),
                    "bytes": int(nbytes), "achieved_gbs": round(nbytes / t / 1e9, 1),
                    "frac": round(nbytes / t / 1e9 / peak, 3)})
    eng.assemble(u1, u0)  # leave the engine's outputs as one assembly left them
    return out


# --------------------------------------------------------------------------- GPU arm


def _time_replay(eng, steps, warmup):
    import torch

    for _ in range(warmup):
        eng.replay()
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(s)
    for _ in range(steps):
        eng.replay()
    b.record(s)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


MLP_FLOPS_PER_SAMPLE = 2 * (8 * 64 + 64 * 64 + 64 * 64 + 64)  # algorithmic: inputs 8 -> 64 -> 64 -> 64 -> 1


def _bf16_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["bf16_tflops"]), "measured"
    return 1900.0, "fallback"


def mlp_scoring(pr, sizes, steps, warmup, dev):
    """Pruning-network scoring time per launch (CUDA events) on both tensor-core
    kernels, on seeded feature rows in the ranges the geometry produces; the
    tcgen05 figure carries a tensor roofline against the measured bf16 peak."""
    import torch

    peak, kind = _bf16_peak()
    out = {}
    for n in sizes:
        rng = np.random.default_rng(11)
        X = np.zeros((n, 8), np.float32)
        X[:, 0] = rng.uniform(0.5, 8.0, n)
        X[:, 1] = rng.uniform(0.0, 1.0, n)
        X[:, 2] = rng.uniform(1.0, 6.0, n)
        X[:, 5] = rng.uniform(-2.0, 8.0, n)
        feat = torch.as_tensor(X.ravel(), device=dev)
        row = {}
        for b in ("mma", "tcgen05"):
            for _ in range(warmup):
                pr.logits(feat, n, backend=b)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(steps):
                pr.logits(feat, n, backend=b)
            e1.record()
            torch.cuda.synchronize()
            row[f"{b}_us"] = 1e3 * e0.elapsed_time(e1) / steps
        if pr.tcgen05_failed():
            row["tcgen05_failed"] = True
        tf = n * MLP_FLOPS_PER_SAMPLE / (row["tcgen05_us"] * 1e-6) / 1e12
        row["tcgen05_tflops"] = tf
        row["tcgen05_frac_of_" + kind + "_bf16"] = tf / peak
        row["speedup_vs_mma_sync"] = row["mma_us"] / row["tcgen05_us"]
        out[str(n)] = row
        del feat
    return out


def pruning_section(args, dev, w, u0, u1, ms_fp64):
    """The mixed assembly with the learned candidate pruning, per Newton iteration.

    The network is trained here, on the GPU, on exact-path labels of 7- and
    37-wire strands; the first detection of the workload is verified exactly
    (missed contacts are reported; the verification puts any back, so R is unchanged).
    """
    import dataclasses

    import torch

    from xkgpu import prune as P
    from xkgpu import workloads as W
    from xkgpu.engine import AssemblyEngine

    t0 = time.perf_counter()
    pr = P.PairPruner(device=dev)
    feats, ys = [], []
    # 7- and 37-wire strands at the benchmark configurations' discretisation and at the 1027-wire one
    # (d 0.5 mm, pitch 20 mm, 24 elements per pitch)
    train = [(lambda sd: W.config_workload("strand7", seed=sd), range(4)),
             (lambda sd: W.config_workload("strand37", seed=sd), range(3)),
             (lambda sd: W.strand_workload("strand7_d05", 7, 0.5, 20.0, 2, 24, seed=sd), range(4)),
             (lambda sd: W.strand_workload("strand37_d05", 37, 0.5, 20.0, 2, 24, seed=sd), range(3))]
    for make_w, seeds in train:
        for sd in seeds:
            ww = make_w(sd)
            e = AssemblyEngine(ww.strand.coords, ww.strand.conn, ww.strand.radii, ww.section, precision="fp64",
                               device=dev, **ww.engine_kwargs())
            rng = np.random.default_rng(100 + sd)
            mask = np.tile([1, 1, 1, 0, 0, 0], ww.strand.n_nodes)
            ua = torch.as_tensor(ww.u, device=dev)
            ub = torch.as_tensor(ww.u + rng.normal(0.0, 3e-3 * ww.meta["d"], ww.u.shape) * mask, device=dev)
            f, y, _ = P.candidate_samples(e, ua, ub, pr)
            feats.append(f)
            ys.append(y)
            del e
    rep = pr.fit(torch.cat(feats), torch.cat(ys), epochs=400)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    st = w.strand
    # the same first Newton iteration without and with pruning, on fresh engines
    ref = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision="mixed", device=dev,
                         **w.engine_kwargs())
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ref.detect(u0)
    torch.cuda.synchronize()
    t_det_ref = time.perf_counter() - t0
    ref.assemble(u1, u0)
    R_ref = ref.R.clone()
    n_ref = ref.pairs.n
    del ref
    eng = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision="mixed", device=dev,
                         **w.engine_kwargs())
    eng.set_pruner(pr, verify_every=10)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    stats = eng.detect(u0)  # the first detection is a verified one
    torch.cuda.synchronize()
    t_det = time.perf_counter() - t0
    eng.assemble(u1, u0)
    R_diff = float((eng.R - R_ref).abs().max() / R_ref.abs().max())
    eng.capture(u1, u0)
    ms = _time_replay(eng, args.steps, args.warmup)
    ps = eng.prune_stats
    out = {"ms_per_step": ms, "speedup_vs_fp64_plain_per_iteration": ms_fp64 / ms,
           "pairs_in_table": eng.pairs.n, "candidates": stats["candidates"],
           "kept_fraction": ps["kept"] / max(ps["candidates"], 1), "verified_detections": ps["verified"],
           "missed_contacts": ps["missed"], "members": stats["members"], "pairs_without_pruning": n_ref,
           "detect_ms_verified": 1e3 * t_det, "detect_ms_without_pruning": 1e3 * t_det_ref,
           "R_rel_diff_vs_unpruned": R_diff, "train_s": t_train, "train": dataclasses.asdict(rep),
           "verify_every": eng.verify_every}
    out["scoring"] = mlp_scoring(pr, (stats["candidates"], 8_000_000), 20, 3, dev)
    del eng
    torch.cuda.empty_cache()
    return out, pr


def detection_section(dev, w, u0, reps: int = 3) -> dict:
    """Per-phase wall times (ms, host-synchronised) of a steady-state detection of the mixed engine
    (merging into an existing table), and the whole detection of both engines."""
    import ctypes as C

    import torch

    from xkgpu import _lib as L
    from xkgpu.device import ptr, stream_handle
    from xkgpu.engine import AssemblyEngine

    st = w.strand
    out = {}
    for prec in ("mixed", "fp64"):
        eng = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision=prec, device=dev,
                             **w.engine_kwargs())
        eng.detect(u0)
        eng.assemble(u0, u0)
        tot = []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            stats = eng.detect(u0)
            torch.cuda.synchronize()
            tot.append(1e3 * (time.perf_counter() - t0))
        res = {"detect_ms": min(tot), "pairs": stats["pairs"], "narrowphase_exact_pairs": stats["narrowphase_exact"]}
        if prec == "mixed":
            s = stream_handle(None)
            ph = {}

            def tic():
                torch.cuda.synchronize()
                return time.perf_counter()

            for _ in range(reps):
                eng.sync_state()
                t = tic()
                cands, nc = eng.candidates(u0)
                t1 = tic()
                eng._spare.reserve(max(eng._spare.cap, eng.pairs.n + nc), keep=False)
                L.call("xk_pairs_merge", C.byref(eng.mesh.c), C.byref(eng.pairs.c), ptr(cands), nc,
                       C.byref(eng._spare.c), s)
                eng._spare.set_n(eng._spare.c.n)
                eng.pairs, eng._spare = eng._spare, eng.pairs
                t2 = tic()
                L.call("xk_nodes_prepare", C.byref(eng.mesh.c), ptr(u0), ptr(u0), ptr(eng.node32), s)
                L.call("xk_narrowphase_screened", C.byref(eng.mesh.c), C.byref(eng.pairs.c), ptr(u0),
                       ptr(eng.node32), C.byref(eng.cp), ptr(eng._n_exact), s)
                t3 = tic()
                eng.pattern.build(eng.pairs)
                t4 = tic()
                eng._to32(s)
                t5 = tic()
                for k, v in (("broadphase", t1 - t), ("merge", t2 - t1), ("narrowphase", t3 - t2),
                             ("pattern", t4 - t3), ("float_table", t5 - t4)):
                    ph[k] = min(ph.get(k, 1e9), 1e3 * v)
            res["phases_ms"] = {k: round(v, 3) for k, v in ph.items()}
        out[prec] = res
        del eng
        torch.cuda.empty_cache()
    return out


def c5_section(args, dev, w, pr) -> dict:
    """The 1027-wire strand through a prescribed bending oscillation (curvature 1/(50 D) cos(2 pi k / 30),
    30 steps, a fresh 3e-4 d jitter per step): every step one detection and two graph-replayed
    Newton-iteration assemblies, with the trained pruner (verified exactly every 10 detections) and
    without it."""
    import torch

    from xkgpu import runs

    st = w.strand
    D = 2.0 * max(x.lay_radius for x in st.wires) + w.meta["d"]
    kappa0 = 1.0 / (50.0 * D)
    n_steps = 30
    out = {"workload": f"{args.workload}: arc of curvature kappa0 cos(2 pi k / {n_steps}), kappa0 = 1/(50 D), "
                       f"D = {D:.2f} mm; seeded noise + 3e-4 d jitter per step", "steps": n_steps}
    res = {}
    for name, p in (("unpruned", None), ("pruned", pr)):
        r = runs.run_detection_oscillation(w, kappa0, n_steps=n_steps, iterations=2, pruner=p, verify_every=10)
        res[name] = r
        torch.cuda.empty_cache()
    a, b = res["unpruned"], res["pruned"]
    ps = b["prune_stats"]
    out["missed_contacts"] = ps["missed"]
    out["verified_detections"] = ps["verified"]
    out["kept_fraction"] = ps["kept"] / max(ps["candidates"], 1)
    out["kept_fraction_per_step"] = [round(k / max(c, 1), 4) for k, c in zip(b["kept_candidates"], b["candidates"])]
    out["members_equal_every_step"] = a["members"] == b["members"]
    for name, r in res.items():
        det = r["detect_ms"][1:]  # the first detection also sizes the buffers
        asm = r["assemble_ms"][1:]
        # detections 0, 10, 20 of the pruned run verify the pruner exactly (the first is left out with the
        # buffer sizing); phase means over the others
        verified = {k for k in range(1, len(det) + 1) if k % 10 == 0} if name == "pruned" else set()
        plain = [p for k, p in enumerate(r["phases_ms"]) if k >= 1 and k not in verified]
        out[name] = {"detect_ms_mean": float(np.mean(det)), "assemble_ms_mean": float(np.mean(asm)),
                     "detect_ms_mean_unverified": float(np.mean([d for k, d in enumerate(det, start=1)
                                                                 if k not in verified])),
                     "phases_ms_mean": {k: round(float(np.mean([p[k] for p in plain])), 3) for k in plain[0]},
                     "pairs_mean": float(np.mean(r["pairs"][1:])),
                     "increment_ms (detection + 2 iterations)": float(np.mean(det) + 2 * np.mean(asm))}
    out["gain_per_increment"] = (out["unpruned"]["increment_ms (detection + 2 iterations)"]
                                 / out["pruned"]["increment_ms (detection + 2 iterations)"])
    out["gain_per_iteration"] = out["unpruned"]["assemble_ms_mean"] / out["pruned"]["assemble_ms_mean"]
    # Newton iterations per increment above which the pruned increment is the cheaper one
    d_det = out["pruned"]["detect_ms_mean"] - out["unpruned"]["detect_ms_mean"]
    d_asm = out["unpruned"]["assemble_ms_mean"] - out["pruned"]["assemble_ms_mean"]
    out["break_even_iterations_per_increment"] = d_det / d_asm if d_asm > 0 and d_det > 0 else (0.0 if d_det <= 0 else None)
    out["R_rel_diff_last_step"] = float((b["R_last"] - a["R_last"]).abs().max() / a["R_last"].abs().max())
    return out


def c2_section(args, dev) -> dict:
    """The 37-wire quasi-static load step: the outer layer pressed radially inward by the lay gap plus
    0.005 d, FP64 and mixed, over the restated solver loop with the device block solve."""
    import torch

    from xkgpu import runs
    from xkgpu import solver as S
    from xkgpu import workloads as W

    out = {}
    us = {}
    for prec in ("fp64", "mixed"):
        w = W.strand_workload("strand37", 37, 2.0, 40.0, 4, 32, gap_frac=0.0, seed=2)
        lay = max(x.lay_radius for x in w.strand.wires) / 3.0 - w.meta["d"]
        amount = lay + 0.005 * w.meta["d"]
        res, b, secs = runs.run_load_step(w, prec, layer=3, amount=amount,
                                          settings=S.SolverSettings(dt_max_fraction=0.1, max_increments=80))
        out[prec] = {"converged": res.converged, "increments": res.n_increments, "newton_attempts": res.total_attempts,
                     "cutbacks": res.n_cutbacks, "wall_s": secs, "solver": dict(getattr(b, "lin_stats", {})),
                     "active_pairs_end": res.increments[-1].n_active if res.increments else 0}
        us[prec] = res.u.cpu().numpy()
        torch.cuda.empty_cache()
    out["workload"] = ("strand37 (37 wires, d 2 mm, pitch 40 mm, 4 pitches, 32 el/pitch, lay gap "
                       f"{lay:.4f} mm): outer layer moved radially inward by {amount:.4f} mm, inner wires clamped "
                       "at both ends")
    out["u_rel_diff_mixed_vs_fp64"] = float(np.abs(us["mixed"] - us["fp64"]).max() / np.abs(us["fp64"]).max())
    return out


def _c3_run(nw: int, n_pitches: int, n_steps: int, max_increments: int = 0) -> dict:
    """One bend-and-release run of the reference's solver loop in FP64, then in mixed precision on the FP64
    run's increments; displacements compared at every common increment and at the end of every step."""
    import torch

    from xkgpu import runs
    from xkgpu import solver as S
    from xkgpu import workloads as W

    w = W.strand_workload(f"strand{nw}", nw, 2.0, 40.0, n_pitches, 32, gap_frac=0.0, seed=0, penalty="beam_ei")
    D = 2.0 * max(x.lay_radius for x in w.strand.wires) + w.meta["d"]
    cfg = dict(dt_min_fraction=1e-3, max_nr_attempts=100, use_line_search=False, max_increments=max_increments,
               tol_force=1e-6)
    kw = dict(kappa=1.0 / (50.0 * D), n_steps=n_steps, bend_time=2e-3,
              bend_settings=S.SolverSettings(dt_max_fraction=0.05, **cfg), step_settings=S.SolverSettings(**cfg))
    out, res = {}, {}
    follow = None
    for prec in ("fp64", "mixed"):
        r = runs.run_bend_oscillation(w, prec, follow=follow, **kw)
        follow = r["schedule"] if follow is None else follow
        n_it = r["counts"]["assemble"]
        out[prec] = {"completed": r["converged"], "bend": {k: r["bend"][k] for k in ("increments", "attempts", "cutbacks",
                                                                                      "converged")},
                     "bend_reached": r["bend"]["load_frac"][-1] if r["bend"]["load_frac"] else 0.0,
                     "steps_done": len(r["step_s"]), "newton_iterations": n_it,
                     "attempts_per_step": [sum(a) for a in r["attempts"][1:]],
                     "ms_per_newton_iteration": 1e3 * r["wall_s"] / max(n_it, 1),
                     "ms_per_iteration_without_linear_solve": 1e3 * (r["wall_s"] - r["solve_s"]) / max(n_it, 1),
                     "wall_s": r["wall_s"], "linear_solve_s": r["solve_s"], "linear_solver": r.get("lin")}
        res[prec] = r
        torch.cuda.empty_cache()
    a, b = res["fp64"], res["mixed"]
    fa = {round(f, 12): k for k, f in enumerate(a["bend"]["load_frac"])}
    common = [(fa[round(f, 12)], k) for k, f in enumerate(b["bend"]["load_frac"]) if round(f, 12) in fa]
    db = [float(np.abs(b["bend_u"][kb] - a["bend_u"][ka]).max() / max(np.abs(a["bend_u"][ka]).max(), 1e-300))
          for ka, kb in common]
    n = min(len(a["u"]), len(b["u"]))
    ds = [float(np.abs(b["u"][k] - a["u"][k]).max() / max(np.abs(a["u"][k]).max(), 1e-300)) for k in range(n)]
    out["workload"] = (f"strand{nw}: {nw} wires, d 2 mm, pitch 40 mm, {n_pitches} pitch(es), 32 el/pitch, at the "
                       f"minimum safe lay gap; bent over 2 ms of Generalized-alpha (rho_inf 0.9) to curvature "
                       f"1/(50 D), D = {D:.2f} mm, then released for {n_steps} steps of 1e-4 s; mu 0.1; k_pen = "
                       f"0.1 * 12 EI / L^3 = {w.k_pen:.4g} N/mm (the reference's default penalty); line search off, at "
                       f"most 100 attempts, force tolerance 1e-6; mixed follows the FP64 run's increments")
    out["u_rel_diff_mixed_vs_fp64"] = {"bend_increments": db, "max_bend": max(db) if db else None,
                                       "steps": ds, "max_steps": max(ds) if ds else None}
    return out


def c3_section(args, dev) -> dict:
    """The 91-wire configuration's bending run (Generalized-alpha bend to curvature 1/(50 D), then 20 steps of
    free oscillation, mu 0.1, graph-replayed assembly, device block solve), FP64 and mixed, on the strand of
    the configuration (91 wires, 4 pitches, as far as the reference's loop carries it: 14 increments at most)
    and in full on a 19-wire strand of one pitch."""
    return {"strand91": _c3_run(91, 4, 20, max_increments=14), "strand19_full": _c3_run(19, 1, 20)}


def batch_section(args, dev):
    """The 256-strand batch (one friction coefficient per strand) assembled by the same launches, with
    the tangent schedule and then the launch shapes chosen by the engine's autotuner."""
    import torch

    from xkgpu import _lib as L
    from xkgpu import workloads as W
    from xkgpu.engine import AssemblyEngine

    w = W.config_workload("batch256", seed=0)
    st = w.strand
    u0 = torch.as_tensor(w.u, device=dev)
    rng = np.random.default_rng(7)
    du = rng.normal(0.0, 2e-4 * w.meta["d"], (st.n_nodes, 6))
    du[:, 3:] = 0.0
    u1 = torch.as_tensor(w.u + du.ravel(), device=dev)
    out = {"workload": "batch256: 256 strands, wires from {7, 19, 37}, 1-4 pitches, 8-48 el/pitch, d = 2 mm, "
                       "gap -0.005 d, seeded noise, mu per strand in [0.05, 0.3]",
           "n_nodes": st.n_nodes, "n_elems": st.n_elems}
    for prec in ("fp64", "mixed"):
        eng = AssemblyEngine(st.coords, st.conn, st.radii, w.section, layer=st.elem_layer, precision=prec,
                             k_pen=w.k_pen, mu=w.mu, device=dev)
        stats = eng.detect(u0)
        eng.capture(u1, u0)  # the tangent schedule is tuned here; the launch shapes keep their defaults
        ms = _time_replay(eng, args.steps, args.warmup)
        units = st.n_elems + stats["pairs"]
        names = {L.XK_GATHER_LANES: "lanes", L.XK_GATHER_CHUNKS: "chunks", L.XK_GATHER_SIDES: "sides"}
        res = {"ms_per_step": ms, "evals_per_s": units / ms * 1e3, "pairs": stats["pairs"],
               "members": stats["members"], "schedule": names.get(eng.gather_variant, "default"),
               "schedule_ms": {names[v]: round(t, 4) for v, t in getattr(eng, "tune_times", {}).items()}}
        # the autotuner over the launch shapes as well: the pair kernels' CTA size and the block gather's
        # persistent CTAs per SM, each timed on this workload; the step with the chosen shapes
        eng.tune(shapes=True)
        eng.capture(u1, u0)
        ms_t = _time_replay(eng, args.steps, args.warmup)
        res["launch_shapes"] = eng.tune_shapes
        res["ms_per_step_tuned_shapes"] = ms_t
        res["gain_tuned_shapes_vs_default"] = ms / ms_t
        out[prec] = res
        del eng
        torch.cuda.empty_cache()
    out["speedup_mixed_vs_fp64"] = out["fp64"]["ms_per_step"] / out["mixed"]["ms_per_step"]
    return out


def coated_section(args, dev):
    """The 91-wire strand with coated wires (core radius 0.9 r; coating stiffness 1e4 N/mm, damping 50,
    coating friction 0.2): every candidate pair is a member and carries the fused coating epilogue.
    (At strand1027 every candidate pair as a member gives contact rows with more than 256 blocks, the
    contact pattern's row limit.)"""
    import torch

    from xkgpu import workloads as W
    from xkgpu.engine import AssemblyEngine

    w = W.config_workload("strand91", seed=0)
    st = w.strand
    r = float(st.radii[0])
    coat = dict(stiffness=1e4, damping=50.0, mu=0.2, k_t_ratio=0.5, dt=0.1)
    u0 = torch.as_tensor(w.u, device=dev)
    rng = np.random.default_rng(11)
    du = rng.normal(0.0, 2e-4 * w.meta["d"], (st.n_nodes, 6))
    du[:, 3:] = 0.0
    u1 = torch.as_tensor(w.u + du.ravel(), device=dev)
    out = {"workload": "strand91 (91 wires, d = 2 mm, 4 pitches, 32 el/pitch) with coated wires (core 0.9 r, "
                       "k 1e4, c 50, coating mu 0.2, dt 0.1)", "n_elems": st.n_elems}
    R = {}
    for prec in ("fp64", "mixed"):
        eng = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision=prec, device=dev,
                             core_radii=0.9 * r, coating=coat, **w.engine_kwargs())
        stats = eng.detect(u0)
        eng.end_step()
        eng.capture(u1, u0)
        ms = _time_replay(eng, max(5, args.steps // 4), args.warmup)
        units = st.n_elems + stats["pairs"]
        out[prec] = {"ms_per_step": ms, "evals_per_s": units / ms * 1e3, "pairs": stats["pairs"],
                     "members": stats["members"], "contact_blocks": stats["contact_blocks"],
                     "contact_blocks_full_matrix": stats["contact_blocks_full"]}
        R[prec] = eng.R.double().cpu().numpy()
        del eng
        torch.cuda.empty_cache()
    out["speedup_mixed_vs_fp64"] = out["fp64"]["ms_per_step"] / out["mixed"]["ms_per_step"]
    out["R_err_mixed_vs_fp64"] = float(np.max(np.abs(R["mixed"] - R["fp64"])) / np.max(np.abs(R["fp64"])))
    return out


def device_solve_section(args, dev):
    """Newton increments with the linear solve on the device against scipy's direct solve.

    The 7-wire strand with its initial penetration relaxed to equilibrium (frictionless, k_pen 1e4 N/mm,
    both wire ends clamped), FP64, the well-posed increment of the Newton tests: ``solve_increment(graph=True, solver=DeviceLinearSolver)`` keeps
    the iteration on the device (assembly graph, block-Jacobi BiCGStab, update), the other run solves
    each Newton step with ``scipy.sparse.linalg.spsolve`` on the host.  One untimed increment first.
    """
    import torch

    from xkgpu import workloads as W
    from xkgpu.engine import AssemblyEngine
    from xkgpu.newton import solve_increment
    from xkgpu.solve import DeviceLinearSolver

    w = W.config_workload("strand7", seed=0)
    st = w.strand
    kw = w.engine_kwargs()
    kw.update(k_pen=1e4, mu=0.0)
    npw = st.n_elems_per_wire + 1
    fixed = np.zeros((st.n_nodes, 6), dtype=bool)
    for wi in range(len(st.wires)):
        fixed[wi * npw] = True
        fixed[wi * npw + npw - 1] = True
    fixed = fixed.ravel()
    out = {"workload": "strand7 (7 wires, 119 nodes, 714 DOFs), frictionless, k_pen 1e4 N/mm, clamped ends, "
                       "FP64; one Newton increment from the initial penetration to equilibrium (tol 1e-9)"}
    u_ref = {}
    for name in ("device", "host"):
        eng = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision="fp64", device=dev, **kw)
        u0 = torch.zeros(eng.mesh.ndof, dtype=torch.float64, device=dev)
        ds = DeviceLinearSolver(eng, rtol=1e-10, max_iter=2000) if name == "device" else None
        try:
            for rep in range(2):
                if ds is not None:
                    ds.history.clear()
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                res = solve_increment(eng, u0, u0, fixed=fixed, tol=1e-9, max_iter=25, solver=ds,
                                      graph=ds is not None)
                torch.cuda.synchronize()
                t = time.perf_counter() - t0
        except Exception as exc:  # noqa: BLE001 - reported in the bench line
            out[name] = {"error": f"{type(exc).__name__}: {exc}"[:300]}
            continue
        u_ref[name] = res.u.cpu().numpy()
        rec = {"converged": res.converged, "newton_iterations": res.iterations, "ms_per_increment": 1e3 * t,
               "ms_per_newton_iteration": 1e3 * t / max(res.iterations, 1)}
        if ds is not None and ds.history:
            its = [h[0] for h in ds.history]
            rec.update(bicgstab_iterations_per_solve=float(np.mean(its)), solves=len(its))
        out[name] = rec
    if "device" in u_ref and "host" in u_ref:
        a, b = u_ref["device"], u_ref["host"]
        out["u_rel_diff_device_vs_host"] = float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
        if "ms_per_increment" in out["device"] and "ms_per_increment" in out["host"]:
            out["speedup_device_vs_host"] = out["host"]["ms_per_increment"] / out["device"]["ms_per_increment"]
    return out


def rank_aggregate(t_max, n_sum, device=None):
    """Times maxed and unit counts summed over the ranks of the default process group.

    One rank (or no process group): the values as given.  The bench's value is
    the units of all ranks over the slowest rank's time.
    """
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(x) for x in t_max], [float(x) for x in n_sum]
    a = torch.tensor([float(x) for x in t_max], dtype=torch.float64, device=device)
    b = torch.tensor([float(x) for x in n_sum], dtype=torch.float64, device=device)
    dist.all_reduce(a, op=dist.ReduceOp.MAX)
    dist.all_reduce(b, op=dist.ReduceOp.SUM)
    return a.tolist(), b.tolist()


def run_gpu(args, rank, world):
    import torch

    from xkgpu import _lib as L
    from xkgpu import workloads as W
    from xkgpu.engine import AssemblyEngine

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    w = W.config_workload(args.workload, seed=rank)
    st = w.strand
    n_e = st.n_elems

    def make(prec):
        return AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision=prec, device=dev,
                              **w.engine_kwargs())

    u0 = torch.as_tensor(w.u, device=dev)
    rng = np.random.default_rng(100 + rank)
    du = rng.normal(0.0, 2e-4 * w.meta["d"], (st.n_nodes, 6))
    du[:, 3:] *= 0.0
    u1 = torch.as_tensor(w.u + du.ravel(), device=dev)

    results = {}
    engines = {}
    for prec in ("fp64", "mixed"):
        eng = make(prec)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        stats = eng.detect(u0)
        torch.cuda.synchronize()
        t_det_first = time.perf_counter() - t0
        t0 = time.perf_counter()
        eng.detect(u0)  # steady state: merge into an existing table
        torch.cuda.synchronize()
        t_det = time.perf_counter() - t0
        eng.capture(u1, u0)
        for _ in range(args.warmup):
            eng.replay()
        torch.cuda.synchronize()
        engines[prec] = eng
        results[prec] = {"stats": stats, "detect_ms": 1e3 * t_det, "detect_first_ms": 1e3 * t_det_first}

    # error of mixed against FP64 on the same state (fresh engines)
    e64, emx = make("fp64"), make("mixed")
    e64.detect(u0)
    emx.detect(u0)
    e64.assemble(u1, u0)
    emx.assemble(u1, u0)
    emx.sync_state()
    torch.cuda.synchronize()

    def relmax(a, b):
        a, b = a.double(), b.double()
        return float((a - b).abs().max() / b.abs().max().clamp_min(1e-300))

    nb = e64.pattern.nnzb
    err = {"R": relmax(emx.R, e64.R), "K_beam": relmax(emx.K_beam, e64.K_beam),
           "K_contact": relmax(emx.K_c[: 9 * nb], e64.K_c[: 9 * nb]),
           "status_equal_after_iteration": bool(torch.equal(emx.pairs.t["status"][: emx.pairs.n],
                                                e64.pairs.t["status"][: e64.pairs.n]))}

    del e64, emx

    if world > 1:
        torch.distributed.barrier()

    def timed(eng, k):
        s = torch.cuda.current_stream()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(s)
        for _ in range(k):
            eng.replay()
        b.record(s)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3

    with ClockSampler(dev.index if dev.index is not None else 0) as clk:
        t_mixed = timed(engines["mixed"], args.steps)
        t_fp64 = timed(engines["fp64"], args.steps)
    clocks = clk.summary()

    n_c = engines["mixed"].pairs.n
    # every rank assembles its own seeded strand: its units count, the slowest rank sets the time
    (t_mixed, t_fp64), (units,) = rank_aggregate([t_mixed, t_fp64], [n_e + n_c], device=dev)
    ms_mixed = 1e3 * t_mixed / args.steps
    ms_fp64 = 1e3 * t_fp64 / args.steps

    # the float beam beside the pair kernels: its launch capped at a few CTAs per SM (the kernel loops), so
    # that it shares the SMs with them instead of holding every SM for its one wave; the step with each cap
    beam_caps = {}
    em = engines["mixed"]
    if world == 1 and em.beam.chain_ordered:
        base = em.beam.plan.beam_ctas_per_sm
        for per_sm in (1, 2, 3):
            em.beam.plan.beam_ctas_per_sm = per_sm
            em.capture(u1, u0)
            for _ in range(args.warmup):
                em.replay()
            beam_caps[str(per_sm)] = 1e3 * timed(em, args.steps) / args.steps
        em.beam.plan.beam_ctas_per_sm = base
        em.capture(u1, u0)
        beam_caps[str(base) + " (the engine's setting)"] = ms_mixed

    # dominant kernel alone: the fused pair kernel, CUDA events on its stream
    import ctypes as C

    from xkgpu.device import ptr, stream_handle

    def pair_kernel_time(eng, k):
        s = torch.cuda.current_stream()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for _ in range(3):
            eng.pair_step(u1, u0, s)
        torch.cuda.synchronize()
        a.record(s)
        for _ in range(k):
            eng.pair_step(u1, u0, s)
        b.record(s)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3 / k

    def gather_kernel_time(eng, k):
        s = torch.cuda.current_stream()
        sh = stream_handle(s)
        args_ = (C.byref(eng.pattern.c), ptr(eng.rec), eng.precision, L.XK_OUT_COMBINED, L.XK_WHICH_COMBINED,
                 eng.gather_variant, ptr(eng.K_c), sh)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for _ in range(3):
            L.call("xk_contact_gather_tangent", *args_)
        torch.cuda.synchronize()
        a.record(s)
        for _ in range(k):
            L.call("xk_contact_gather_tangent", *args_)
        b.record(s)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3 / k

    kreps = max(20, min(args.steps, 200))
    tk_mixed = pair_kernel_time(engines["mixed"], kreps)
    tk_fp64 = pair_kernel_time(engines["fp64"], kreps)
    tg_mixed = gather_kernel_time(engines["mixed"], kreps)
    tg_fp64 = gather_kernel_time(engines["fp64"], kreps)
    pat = engines["mixed"].pattern
    m = pat.n_members
    by_mixed = pair_kernel_bytes(st.n_nodes, n_e, n_c - m, m, True)
    by_fp64 = pair_kernel_bytes(st.n_nodes, n_e, n_c - m, m, False)
    sides = (L.XK_GATHER_SIDES,)
    bg_mixed = gather_tangent_bytes(m, pat.n_contrib, pat.nnzb, True, engines["mixed"].gather_variant in sides, n_e)
    bg_fp64 = gather_tangent_bytes(m, pat.n_contrib, pat.nnzb, False, engines["fp64"].gather_variant in sides, n_e)
    variant_name = {L.XK_GATHER_LANES: "lanes", L.XK_GATHER_CHUNKS: "chunks", L.XK_GATHER_SIDES: "sides"}
    kernel_names = {L.XK_GATHER_LANES: "k_gather_tangent_lanes<float>", L.XK_GATHER_CHUNKS: "k_gather_tangent<float>",
                    L.XK_GATHER_SIDES: "k_elem_sums<float> + k_gather_tangent_sides<float>"}
    peak, peak_kind = _peaks()
    kernels = None
    if engines["mixed"].gather_variant == L.XK_GATHER_SIDES:
        kernels = kernel_roofline_mixed(engines["mixed"], u1, u0, peak)
    # the autotuner's times of every tangent schedule (ms per call), before the engines are released
    sched_ms = {p: {variant_name[v]: round(t, 4) for v, t in getattr(engines[p], "tune_times", {}).items()}
                for p in ("mixed", "fp64")}

    # end to end through the public engine API with host buffers: each step copies u and u_ref in from
    # pinned host memory and reads R, K_beam and K_c back; the read-back of one step overlaps the next
    from xkgpu.engine import HostPipeline

    pipe = HostPipeline(engines["mixed"])
    uh = torch.empty_like(u1, device="cpu").pin_memory()
    uh.copy_(u1.cpu())
    urh = torch.empty_like(u0, device="cpu").pin_memory()
    urh.copy_(u0.cpu())
    for _ in range(args.warmup):
        pipe.result(pipe.submit(uh, urh))
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(s)
    prev = None
    for _ in range(args.steps):
        k = pipe.submit(uh, urh)
        if prev is not None:
            pipe.result(prev)  # the host holds step k-1's R and K while step k runs
        prev = k
    pipe.result(prev)
    s.wait_stream(pipe.copy_out)
    b.record(s)
    torch.cuda.synchronize()
    t_e2e = a.elapsed_time(b) / 1e3
    (t_e2e,), _ = rank_aggregate([t_e2e], [], device=dev)
    h2d = pipe.bytes_in
    d2h = pipe.bytes_out
    del pipe
    # the same round trip for a caller whose linear solve stays on the device: R and its norm come back
    lean = HostPipeline(engines["mixed"], read_tangent=False)
    for _ in range(args.warmup):
        lean.result(lean.submit(uh, urh))
    torch.cuda.synchronize()
    a.record(s)
    prev = None
    for _ in range(args.steps):
        k = lean.submit(uh, urh)
        if prev is not None:
            lean.result(prev)
        prev = k
    lean.result(prev)
    s.wait_stream(lean.copy_out)
    b.record(s)
    torch.cuda.synchronize()
    t_lean = a.elapsed_time(b) / 1e3
    (t_lean,), _ = rank_aggregate([t_lean], [], device=dev)
    d2h_lean = lean.bytes_out
    del lean

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        frac = 1.0 / 48.0
        _, dt, prep = oracle_sample_timing(w, frac)  # includes a warm first call
        units_c, dt, _ = oracle_sample_timing(w, frac, reps=1, prepared=prep)
        sub = prep[0]
        cpu = {"value": units_c / dt, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"NumPy oracle, one Newton-iteration assembly (contact + beam) on the first 1/48 of every "
                         f"wire ({sub.n_elems} elements, {prep[2]['ea'].shape[0]} pairs), host cores of the machine that runs the bench"}

    mixed_variant = engines["mixed"].gather_variant
    beam_launches = 1 if engines["mixed"].beam.chain_ordered else 2
    fp64_variant = engines["fp64"].gather_variant
    contact_blocks = engines["mixed"].pattern.nnzb
    contact_blocks_full = engines["mixed"].pattern.nnzb_full
    extras = {}
    if not args.no_extras and world == 1:
        del engines, eng
        torch.cuda.empty_cache()
        extras["detection"] = detection_section(dev, w, u0)
        extras["learned_pruning"], pr = pruning_section(args, dev, w, u0, u1, ms_fp64)
        extras["c5_oscillation"] = c5_section(args, dev, w, pr)
        del pr
        if args.runs:
            extras["c2_load_step"] = c2_section(args, dev)
            extras["c3_oscillation"] = c3_section(args, dev)
        extras["batched"] = batch_section(args, dev)
        extras["coated"] = coated_section(args, dev)
        extras["device_solve"] = device_solve_section(args, dev)

    # node prep, the other-pair kernel and its near-parallel kernel, the beam (one launch for wires whose
    # elements follow each other; a zeroing launch before it for other chain meshes), the member kernel
    # and its near-parallel kernel, then either element sums + tangent gather + residual from the element
    # sums (norm fused) or tangent gather + force gather + 2 norm kernels (an ncu launch list of one
    # replayed step shows the nine launches of the first form on the strand)
    per_launch = 5 + beam_launches + (3 if mixed_variant == L.XK_GATHER_SIDES else 4)
    out = {
        "metric": METRIC, "value": units / t_mixed * args.steps, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_mixed, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (mixed: float arithmetic and float quaternion frames; float-float contact gap of contributing pairs; FP64 near-parallel closest points, detection decisions near the thresholds and residual norm)",
        "data": "synthetic (seeded strand geometry and perturbations of the reference's configuration)",
        "config": {"workload": "strand1027: 1027 wires (18 layers), d=0.5 mm, pitch 20 mm, 4 pitches, "
                               "24 el/pitch, gap -0.005 d, seeded noise", "n_nodes": st.n_nodes,
                   "n_elems": n_e, "n_pairs": n_c, "raw_aabb_pairs": results["mixed"]["stats"]["raw"],
                   "contributing_pairs": m, "contact_blocks": contact_blocks,
                   "contact_blocks_full_matrix": contact_blocks_full,
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (pair table alone > 1 GB)", "cuda_graph": True},
        "beam_ctas_per_sm_ms_per_step": beam_caps,
        "fp64_plain": {"value": units / t_fp64 * args.steps, "ms_per_step": ms_fp64,
                       "speedup_mixed_vs_fp64": t_fp64 / t_mixed},
        "err_vs_fp64": err,
        "detect_ms": {"mixed": results["mixed"]["detect_ms"], "fp64": results["fp64"]["detect_ms"],
                      "first": results["mixed"]["detect_first_ms"]},
        "roofline": {"bound": "hbm",
                     "kernel": "contact tangent gather, schedule " + variant_name.get(mixed_variant, "default")
                               + " (" + kernel_names.get(mixed_variant, "") + ")",
                     "achieved": bg_mixed / tg_mixed / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": bg_mixed / tg_mixed / 1e9 / peak, "peak_kind": peak_kind,
                     "bytes_per_launch": bg_mixed, "launch_ms": 1e3 * tg_mixed, "traffic": None,
                     "schedule_ms": sched_ms["mixed"],
                     "fp64_kernel": {"achieved": bg_fp64 / tg_fp64 / 1e9, "launch_ms": 1e3 * tg_fp64,
                                     "bytes_per_launch": bg_fp64,
                                     "schedule": variant_name.get(fp64_variant, "default"),
                                     "schedule_ms": sched_ms["fp64"]},
                     "pair_step": {"kernels": "k_nodes_prepare + k_pair_other32 + k_pair_member32 (narrowphase, "
                                              "Huber, Coulomb, pair tangent)",
                                   "achieved": by_mixed / tk_mixed / 1e9, "frac": by_mixed / tk_mixed / 1e9 / peak,
                                   "bytes_per_launch": by_mixed, "launch_ms": 1e3 * tk_mixed,
                                   "fp64": {"achieved": by_fp64 / tk_fp64 / 1e9, "launch_ms": 1e3 * tk_fp64,
                                            "bytes_per_launch": by_fp64}}},
        "kernels_mixed": kernels,
        "e2e": {"value": units / t_e2e * args.steps, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "e2e_residual_only": {"value": units / t_lean * args.steps, "unit": UNIT, "h2d_bytes_per_step": h2d,
                              "d2h_bytes_per_step": d2h_lean,
                              "note": "the same round trip reading back R and its FP64 norm only (K_beam and K_c "
                                      "stay on the device for a device linear solve)"},
        "gpu_launches": per_launch * args.steps,
        "clocks": clocks,
        "cpu_baseline": cpu,
        **extras,
    }
    tr = ROOT / "profiles" / "dram_traffic.json"
    if tr.exists():
        d = json.loads(tr.read_text())
        key = {L.XK_GATHER_SIDES: "gather_tangent_sides_float"}.get(mixed_variant)
        out["roofline"]["traffic"] = d.get(key, {}).get("bytes_per_launch") if key else None
        out["roofline"]["pair_step"]["traffic"] = d.get("pair_step_mixed", {}).get("bytes_per_launch")
        out["roofline"]["traffic_source"] = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of a separate "
                                             "capture, recorded in profiles/dram_traffic.json; not measured "
                                             "in this run")
    return out


# --------------------------------------------------------------------------- reference arm


def _ref_worker(conn, workload: str, frac: float, index: int) -> None:
    """One host core's share of the reference arm: slab ``index`` of every wire, prepared once
    (untimed), then one Newton-iteration assembly of it per request."""
    from xkgpu import workloads as W

    w = W.config_workload(workload, seed=0)
    units, dt, prep = oracle_sample_timing(w, frac, index=index)
    conn.send((units, dt))
    while conn.recv() == "step":
        units, dt, _ = oracle_sample_timing(w, frac, prepared=prep)
        conn.send((units, dt))


def run_reference(args):
    """The reference path (the NumPy port) on every host core: one spawned process per core, each
    assembling its own slab of every wire; a step ends when every process has finished its slab."""
    import multiprocessing as mp

    from xkgpu import workloads as W

    w = W.config_workload(args.workload, seed=0)
    budget = float(os.environ.get("XK_REF_BUDGET_S", "150"))
    frac = 1.0 / 96.0
    _, dt0, _ = oracle_sample_timing(w, frac)
    per_step = budget / max(1, args.steps + args.warmup)
    # shrink the slab until one step fits its share of the budget
    while dt0 > per_step and frac > 1.0 / 768.0:
        frac /= 2.0
        _, dt0, _ = oracle_sample_timing(w, frac)
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    nel = w.strand.n_elems_per_wire
    n = max(1, min(cores, nel // slab_elems(nel, frac)))
    for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[var] = "1"  # one thread per process: the processes are the parallelism
    ctx = mp.get_context("spawn")
    pipes, procs = [], []
    for k in range(n):
        a, b = ctx.Pipe()
        pr = ctx.Process(target=_ref_worker, args=(b, args.workload, frac, k), daemon=True)
        pr.start()
        pipes.append(a)
        procs.append(pr)
    slab_units = [a.recv()[0] for a in pipes]  # prepared

    def step():
        for a in pipes:
            a.send("step")
        return sum(a.recv()[0] for a in pipes)

    for _ in range(args.warmup):
        step()
    units = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        units += step()
    tt = time.perf_counter() - t0
    for a in pipes:
        a.send("stop")
    for pr in procs:
        pr.join(timeout=30)
    v = units / tt
    sample = (f"NumPy port of the reference path (oracle) in {n} processes, one per host core, each one "
              f"Newton-iteration assembly per step of its own {frac:.4g} slab of every wire "
              f"({n * slab_elems(nel, frac)} of {nel} elements per wire; {sum(slab_units)} elements + pairs)")
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * tt / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "strand1027 slab sample", "sample_fraction": n * frac, "processes": n},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": n, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_profile(args):
    """Small driver for ncu: one engine, one detection, ``--steps`` eager assemblies."""
    import torch

    from xkgpu import _lib as L
    from xkgpu import workloads as W
    from xkgpu.engine import AssemblyEngine

    if args.profile == "mlp":
        # pruning-network scoring on --mlp-n seeded feature rows, --steps launches of each kernel
        from xkgpu import prune as P

        print(json.dumps({"profile": "mlp", "n": args.mlp_n,
                          "scoring": mlp_scoring(P.PairPruner(), (args.mlp_n,), args.steps, 1, "cuda")}))
        return
    w = W.config_workload(args.workload, seed=0)
    st = w.strand
    eng = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision=args.profile, **w.engine_kwargs())
    u0 = torch.as_tensor(w.u, device="cuda")
    u1 = u0 * 1.001
    for k in range(args.detections):
        # the last detection (steady state: the table merged into itself) in an NVTX range "detect", for
        # ncu --nvtx --nvtx-include "detect/"
        if k == args.detections - 1:
            torch.cuda.synchronize()
            torch.cuda.nvtx.range_push("detect")
        stats = eng.detect(u0)
        if k == args.detections - 1:
            torch.cuda.synchronize()
            torch.cuda.nvtx.range_pop()
    if args.schedule != "auto":  # a fixed tangent schedule (the autotuner's timings are distorted under ncu)
        eng.gather_variant = {"lanes": L.XK_GATHER_LANES, "chunks": L.XK_GATHER_CHUNKS,
                              "sides": L.XK_GATHER_SIDES}[args.schedule]
    eng.assemble(u1, u0)
    if args.schedule == "auto":
        eng.tune()  # the schedule the timed graph uses
    for _ in range(args.steps):
        eng.assemble(u1, u0)
    torch.cuda.synchronize()
    pat = eng.pattern
    print(json.dumps({"profile": args.profile, "workload": args.workload, **stats, "nnzb": pat.nnzb,
                      "n_contrib": pat.n_contrib, "gather_variant": eng.gather_variant,
                      "schedule_ms": {str(k): v for k, v in getattr(eng, "tune_times", {}).items()},
                      "device_bytes_peak": torch.cuda.max_memory_allocated()}))


def run_breakdown(args):
    """Warm per-phase times of one assembly (CUDA events around each phase, eager launches)."""
    import ctypes as C

    import torch

    from xkgpu import _lib as L
    from xkgpu import workloads as W
    from xkgpu.device import ptr, stream_handle
    from xkgpu.engine import AssemblyEngine

    w = W.config_workload(args.workload, seed=0)
    st = w.strand
    out = {"workload": args.workload}
    for prec in ("mixed", "fp64"):
        eng = AssemblyEngine(st.coords, st.conn, st.radii, w.section, precision=prec, **w.engine_kwargs())
        u0 = torch.as_tensor(w.u, device="cuda")
        u1 = u0 * 1.001
        eng.detect(u0)
        p = eng.precision
        s = torch.cuda.current_stream()
        sh = stream_handle(s)
        pat = C.byref(eng.pattern.c)

        def beam():
            if p == L.XK_MIXED:
                L.call("xk_beam_assemble32", C.byref(eng.mesh.c), C.byref(eng.beam.section), ptr(eng.elem32),
                       C.byref(eng.beam.plan), ptr(eng.node32), ptr(eng.f_int), ptr(eng.K_beam), sh)
            else:
                eng.beam.assemble(u1, p, eng.f_int, eng.K_beam, s)

        phases = {
            "pair_step": lambda: eng.pair_step(u1, u0, s),
            "beam": beam,
            "force_gather+norm": lambda: L.call("xk_contact_gather_force", pat, ptr(eng.rec), p, L.XK_OUT_COMBINED,
                                                L.XK_WHICH_COMBINED, ptr(eng.f_int), -1.0, None, None, ptr(eng.R),
                                                ptr(eng.norm2), sh),
            "force_from_elem_sums+norm": lambda: L.call("xk_contact_gather_force_elem", pat, p, ptr(eng.f_int), -1.0,
                                                        None, None, ptr(eng.R), ptr(eng.norm2), sh),
            "tangent_gather_lanes": lambda: L.call("xk_contact_gather_tangent", pat, ptr(eng.rec), p,
                                                   L.XK_OUT_COMBINED, L.XK_WHICH_COMBINED, L.XK_GATHER_LANES,
                                                   ptr(eng.K_c), sh),
            "tangent_gather_chunks": lambda: L.call("xk_contact_gather_tangent", pat, ptr(eng.rec), p,
                                                    L.XK_OUT_COMBINED, L.XK_WHICH_COMBINED, L.XK_GATHER_CHUNKS,
                                                    ptr(eng.K_c), sh),
            "tangent_gather_sides": lambda: L.call("xk_contact_gather_tangent", pat, ptr(eng.rec), p,
                                                   L.XK_OUT_COMBINED, L.XK_WHICH_COMBINED, L.XK_GATHER_SIDES,
                                                   ptr(eng.K_c), sh),
            "assemble": lambda: eng.assemble(u1, u0, stream=s),
        }
        res = {}
        for name, fn in phases.items():
            for _ in range(3):
                fn()
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(s)
            for _ in range(args.steps):
                fn()
            b.record(s)
            torch.cuda.synchronize()
            res[name] = a.elapsed_time(b) / args.steps
        out[prec] = {k: round(v, 4) for k, v in res.items()}
        del eng
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="xkgpu", choices=["xkgpu", "reference"])
    ap.add_argument("--workload", default="strand1027")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the learned-pruning and batched sections")
    ap.add_argument("--runs", action="store_true", help="also the solver runs (37-wire load step, 91-wire bending "
                                                        "oscillation), several minutes")
    ap.add_argument("--mlp-n", type=int, default=8_000_000, help="samples scored by --profile mlp")
    ap.add_argument("--profile", choices=["mixed", "fp64", "mlp"], default=None,
                    help="profiling driver: --detections detections, then --steps eager assemblies, no timing")
    ap.add_argument("--breakdown", action="store_true", help="warm per-phase times (ms) of one assembly")
    ap.add_argument("--schedule", choices=["auto", "lanes", "chunks", "sides"], default="auto",
                    help="tangent schedule of --profile (auto: the autotuner's choice)")
    ap.add_argument("--detections", type=int, default=1,
                    help="detections of --profile; the last one runs in the NVTX range 'detect'")
    args = ap.parse_args()
    if args.breakdown:
        run_breakdown(args)
        return
    if args.profile:
        run_profile(args)
        return
    args.warmup = max(args.warmup, 3)
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)))
        return
    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl")
    out = run_gpu(args, rank, world)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
