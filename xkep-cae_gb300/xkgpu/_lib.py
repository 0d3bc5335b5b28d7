"""ctypes binding of the xkgpu C ABI (``include/xkgpu.h``).

The library is the in-tree ``libxkgpu.so`` built by ``xkgpu.build``.  Loading
fails loudly when it is missing: there is no CPU path behind this module.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libxkgpu.so"

XK_OK, XK_ERR_ARG, XK_ERR_CUDA, XK_ERR_CAPACITY, XK_ERR_OVERFLOW = 0, 1, 2, 3, 4
XK_FP64, XK_MIXED = 0, 1
XK_STAGE_NARROW, XK_STAGE_NORMAL, XK_STAGE_FRICTION, XK_STAGE_TANGENT = 1, 2, 4, 8
XK_STAGE_ALL = 15
XK_STAGE_NO_OTHERS, XK_STAGE_NO_MEMBERS = 16, 32
XK_PAIRS_OTHERS, XK_PAIRS_MEMBERS, XK_PAIRS_ALL = 1, 2, 3
XK_OUT_COMBINED, XK_OUT_SPLIT = 0, 1
XK_WHICH_COMBINED, XK_WHICH_NORMAL, XK_WHICH_FRICTION = 0, 1, 2
REC_STRIDE = {XK_OUT_COMBINED: 16, XK_OUT_SPLIT: 32}
XK_GATHER_DEFAULT, XK_GATHER_LANES, XK_GATHER_CHUNKS, XK_GATHER_SIDES = 0, 1, 2, 3
XK_GATHER_SIDES_SUMS, XK_GATHER_SIDES_BLOCKS = 4, 5
XK_COAT_FORCE, XK_COAT_TANGENT, XK_COAT_FRICTION, XK_COAT_FRICTION_TANGENT = 1, 2, 4, 8

vp = C.c_void_p


class Section(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("E", "G", "A", "Iy", "Iz", "J", "kappa_y", "kappa_z", "scf")]


class StrandSpec(C.Structure):
    _fields_ = [("n_wires", C.c_int32), ("n_elems_per_wire", C.c_int32), ("lay_direction", C.c_int32),
                ("pad", C.c_int32), ("wire_diameter", C.c_double), ("pitch", C.c_double), ("length", C.c_double),
                ("gap", C.c_double), ("x_offset", C.c_double), ("node_first", C.c_int64), ("elem_first", C.c_int64)]


class CoatingState(C.Structure):
    _fields_ = [(n, vp) for n in ("cc", "cc_prev", "z_t", "stick", "q_trial_norm", "dissipation")]


class CoatingParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("stiffness", "damping", "mu", "k_t_ratio", "dt")]


class Mesh(C.Structure):
    _fields_ = [("n_nodes", C.c_int32), ("n_elems", C.c_int32), ("X", vp), ("conn", vp), ("radii", vp),
                ("layer", vp), ("mu", vp), ("core_radii", vp)]


COAT64_FIELDS = ("coat_cc", "coat_cc_prev", "coat_z_t", "coat_qtn", "coat_diss", "coat_stick")
COAT32_FIELDS = ("coat_total", "coat_cc", "coat_cc_prev", "coat_z_t", "coat_qtn", "coat_diss", "coat_stick")


class Pairs(C.Structure):
    _fields_ = [("n", C.c_int32), ("cap", C.c_int32)] + [
        (n, vp) for n in ("ea", "eb", "s", "t", "gap", "normal", "t1", "t2", "lambda_n", "k_pen", "k_t", "p_n",
                          "z_t", "q_trial_norm", "dissipation", "status", "stick")] + [
        (n, vp) for n in COAT64_FIELDS]


class Pairs32(C.Structure):
    _fields_ = [("n", C.c_int32), ("cap", C.c_int32), ("n_members", C.c_int32)] + [
        (n, vp) for n in ("pair", "nodes", "rad", "s", "t", "gap", "normal", "t1", "t2", "p_n", "z_t", "q_trial_norm",
                          "dissipation", "k_pen", "k_t", "status", "stick", "mu")] + [
        (n, vp) for n in COAT32_FIELDS] + [("defer", vp), ("block", C.c_int32), ("pad_launch", C.c_int32),
                                           ("slot", vp)]


class BeamPlan(C.Structure):
    _fields_ = [("n_colors", C.c_int32), ("color_ptr_host", vp), ("elem_order", vp), ("blk", vp), ("first", vp),
                ("nnzb", C.c_int64), ("node_diag", vp), ("chain_ordered", C.c_int32),
                ("beam_ctas_per_sm", C.c_int32)]


class ContactParams(C.Structure):
    _fields_ = [("k_pen", C.c_double), ("k_t_ratio", C.c_double), ("mu_eff", C.c_double),
                ("smoothing_delta", C.c_double), ("g_on", C.c_double), ("g_off", C.c_double),
                ("allow_deactivation", C.c_int32)] + [
        (n, C.c_double) for n in ("coat_k", "coat_c", "coat_mu", "coat_kt_ratio", "coat_dt")]


class System(C.Structure):
    _fields_ = [("n_nodes", C.c_int32), ("precision", C.c_int32)] + [
        (n, vp) for n in ("kb_row_ptr", "kb_col", "kb_vals", "kb_blk_row", "kb_low_ptr", "kb_low_blk", "kc_row_ptr",
                          "kc_col", "kc_vals", "kc_blk_row", "kc_low_ptr", "kc_low_blk", "fixed")]


class BPParams(C.Structure):
    _fields_ = [("margin", C.c_double), ("exclude_shared", C.c_int32), ("exclude_same_layer", C.c_int32),
                ("midpoint_prescreening", C.c_int32), ("prescreening_margin", C.c_double), ("cell_size", C.c_double)]


class ContactPattern(C.Structure):
    _fields_ = [("n_nodes", C.c_int32), ("n_members", C.c_int32), ("n_others", C.c_int32),
                ("nnzb", C.c_int64), ("n_contrib", C.c_int64), ("cap_members", C.c_int64),
                ("cap_others", C.c_int64), ("cap_blocks", C.c_int64)] + [
        (n, vp) for n in ("members", "member_nodes", "others", "inc_ptr", "inc", "row_ptr", "col", "blk_row",
                          "blk_ptr", "contrib")] + [("n_elems", C.c_int64), ("sides_ok", C.c_int64)] + [
        (n, vp) for n in ("node_elem_ptr", "node_elem", "elem_ptr", "elem_inc", "bcodes", "elem_sums",
                          "norm_scratch")] + [("nnzb_full", C.c_int64), ("low_ptr", vp), ("low_blk", vp),
                                              ("sides_per_sm", C.c_int32), ("node_elem_ready", C.c_int32)]


P = C.POINTER
i64p = P(C.c_int64)

# name -> (argtypes); every function returns xk_status (int)
SIGNATURES = {
    "xk_beam_reference": [P(Mesh), P(C.c_double), vp, vp],
    "xk_beam_assemble": [P(Mesh), P(Section), vp, P(BeamPlan), vp, C.c_int, vp, vp, vp],
    "xk_beam_lumped_mass": [P(Mesh), P(Section), P(BeamPlan), C.c_double, vp, vp],
    "xk_broadphase": [P(Mesh), vp, P(BPParams), vp, C.c_int64, i64p, i64p, i64p, vp],
    "xk_pairs_merge": [P(Mesh), P(Pairs), vp, C.c_int64, P(Pairs), vp],
    "xk_pairs_merge_pruned": [P(Mesh), P(Pairs), vp, C.c_int64, P(Pairs), vp],
    "xk_narrowphase": [P(Mesh), P(Pairs), vp, P(ContactParams), C.c_int, vp],
    "xk_narrowphase_screened": [P(Mesh), P(Pairs), vp, vp, P(ContactParams), vp, vp],
    "xk_strand_generate": [vp, C.c_int32, C.c_int64, C.c_int64, vp, vp, vp, vp, vp],
    "xk_pair_gauss_points": [P(Mesh), P(Pairs), vp, C.c_int32, vp, vp],
    "xk_coating_geometry": [P(Pairs), vp, P(ContactParams), C.c_int, vp, vp],
    "xk_coating_step": [P(Pairs), P(ContactPattern), P(CoatingState), vp, vp, P(CoatingParams), C.c_int, vp, vp],
    "xk_contact_pattern_build": [P(Mesh), P(Pairs), P(ContactPattern), vp],
    "xk_pair_step": [P(Mesh), P(Pairs), P(ContactPattern), vp, vp, P(ContactParams), C.c_int, C.c_int, C.c_int, vp,
                     vp],
    "xk_contact_gather_force": [P(ContactPattern), vp, C.c_int, C.c_int, C.c_int, vp, C.c_double, vp, vp, vp, vp,
                                vp],
    "xk_contact_gather_tangent": [P(ContactPattern), vp, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp],
    "xk_contact_gather_force_elem": [P(ContactPattern), C.c_int, vp, C.c_double, vp, vp, vp, vp, vp],
    "xk_constraint_jacobian": [P(Mesh), P(Pairs), vp, vp, vp, vp, C.c_int64, i64p, vp],
    "xk_constraint_jacobian_noalloc": [P(Mesh), P(Pairs), vp, vp, vp, vp, C.c_int64, i64p, vp],
    "xk_norm2": [vp, C.c_int64, vp, vp],
    "xk_softplus_normal_law": [C.c_int64, vp, vp, C.c_double, C.c_double, vp, vp, vp],
    "xk_nodes_prepare": [P(Mesh), vp, vp, vp, vp],
    "xk_beam_prepare32": [P(Mesh), vp, vp, vp],
    "xk_beam_assemble32": [P(Mesh), P(Section), vp, P(BeamPlan), vp, vp, vp, vp],
    "xk_pairs_to32": [P(Mesh), P(Pairs), P(ContactPattern), P(Pairs32), vp],
    "xk_pairs_from32": [P(Pairs32), P(Pairs), vp],
    "xk_pair_step32": [P(Pairs32), vp, P(ContactParams), vp, C.c_int, vp],
    "xk_genalpha_predict": [C.c_int64, vp, vp, vp, vp, vp, vp, vp, C.c_double, C.c_double, C.c_double, vp],
    "xk_genalpha_correct": [C.c_int64, vp, vp, vp, vp, vp, C.c_double, C.c_double, C.c_double, vp],
    "xk_genalpha_residual": [C.c_int64, vp, vp, vp, vp, C.c_double, vp, vp],
    "xk_add_diagonal": [C.c_int64, vp, vp, C.c_double, C.c_int, vp, vp],
    "xk_prune_features": [P(Mesh), vp, vp, C.c_int64, P(Pairs), vp, vp, vp],
    "xk_mlp_forward": [vp, vp, C.c_int64, vp, vp],
    "xk_mlp_forward_tcgen05": [vp, vp, C.c_int64, vp, vp, vp],
    "xk_mlp_train_forward": [vp, vp, C.c_int64, vp, vp, vp],
    "xk_mlp_backward": [vp, vp, vp, vp, vp, vp, C.c_int64, vp, vp, vp, vp, vp],
    "xk_mlp_adam": [vp, vp, vp, vp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, vp, vp],
    "xk_mlp_to_bf16": [vp, vp, vp],
    "xk_prune_select": [vp, C.c_int64, vp, vp, C.c_float, C.c_int, vp, vp, i64p, P(C.c_int32), vp],
    "xk_pairs_drop_pristine": [P(Pairs), vp, C.c_int64, P(Pairs), vp],
    "xk_system_spmv": [P(System), vp, vp, vp],
    "xk_system_block_jacobi": [P(System), vp, vp],
    "xk_bicgstab": [P(System), vp, vp, vp, vp, C.c_int32, C.c_int32, C.c_double, P(C.c_int32), P(C.c_double), vp],
    "xk_system_blocktri": [P(System), vp, C.c_int32, C.c_int32, vp, C.c_double, vp, vp, vp, vp, vp],
}
SOLVE_REDUCE_BLOCKS = 304
MLP_IN, MLP_HIDDEN, MLP_PARAMS, MLP_ACT = 8, 64, 8961, 192
JACOBIAN_NOALLOC_MAX_PAIRS = 1048576
NODE32_STRIDE = 16
ELEM32_STRIDE = 16


class XkError(RuntimeError):
    def __init__(self, code: int, where: str, message: str):
        super().__init__(f"{where}: status {code}: {message}")
        self.code = code


_lib = None


def load() -> C.CDLL:
    """Load ``libxkgpu.so``; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: build the CUDA library first (xkgpu.build.build())")
    lib = C.CDLL(str(LIB_PATH))
    lib.xk_version.restype = C.c_char_p
    lib.xk_last_error.restype = C.c_char_p
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    _lib = lib
    return lib


def exported_symbols() -> list[str]:
    return ["xk_version", "xk_last_error", *SIGNATURES.keys()]


def call(name: str, *args, allow=()) -> int:
    lib = load()
    code = getattr(lib, name)(*args)
    if code != XK_OK and code not in allow:
        raise XkError(code, name, lib.xk_last_error().decode(errors="replace"))
    return code
