/*
 * xkgpu: GPU (sm_103a) assembly of the CR-beam + frictional-contact Newton
 * iteration of the xkep-cae strand solver, as a plain C ABI.
 *
 * All array arguments are DEVICE pointers unless marked "host".  Nothing here
 * takes a framework type: callers pass raw pointers, sizes and a CUDA stream
 * (cudaStream_t cast to void*; NULL is the legacy default stream).  Every
 * function returns an xk_status; xk_last_error() gives a message.
 *
 * Layouts (see the package documentation for byte counts):
 *   u, f, R        double[6*n_nodes], node-major [ux,uy,uz,rx,ry,rz]
 *   beam K_T       block-CSR of 6x6 node blocks, row-major inside a block
 *   contact K_c    block-CSR of 3x3 translational node blocks
 *   pair table     structure of arrays, vector fields component-major with
 *                  stride `cap` (x[c*cap + i])
 */
#ifndef XKGPU_H
#define XKGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int xk_status;
#define XK_OK 0
#define XK_ERR_ARG 1       /* bad argument */
#define XK_ERR_CUDA 2      /* CUDA runtime error */
#define XK_ERR_CAPACITY 3  /* an output buffer is too small; required size is reported */
#define XK_ERR_OVERFLOW 4  /* a bounded per-item work list overflowed */

#define XK_FP64 0   /* every operation in double */
#define XK_MIXED 1  /* float arithmetic and float quaternion frames; contact gaps of contributing pairs in
                       float-float; near-parallel closest points, detection decisions near the
                       thresholds and the residual norm in double */

typedef void* xk_stream;

const char* xk_version(void);
const char* xk_last_error(void);

/* ------------------------------------------------------------------ model */

/* Beam section and material; ULCRBeamAssembler.__init__
 * (xkep_cae/elements/_beam_assembler.py:33-67).  scf <= 0 disables the
 * slenderness compensation of timo_beam3d_ke_local (_beam_cr.py:116-122). */
typedef struct {
  double E, G, A, Iy, Iz, J, kappa_y, kappa_z, scf;
} xk_section;

/* Mesh: reference coordinates, two-node elements, contact radius and layer of
 * every element (DetectCandidatesInput, xkep_cae/contact/_manager_process.py:135-146,
 * and _ContactConfigInput.elem_layer_map, _contact_pair.py:109). */
typedef struct {
  int32_t n_nodes, n_elems;
  const double* X;      /* [3*n_nodes] */
  const int32_t* conn;  /* [2*n_elems] */
  const double* radii;  /* [n_elems] */
  const int32_t* layer; /* [n_elems], -1 = no layer; NULL = no layer map */
  const double* mu;     /* [n_elems] friction coefficient per element (a pair uses mu[ea]: batched strands
                           with their own coefficient, already ramped); NULL = xk_contact_params.mu_eff */
  const double* core_radii; /* [n_elems] or NULL.  Coated wires (set it only when the coating stiffness
                               is positive, as the reference switches on coating_stiffness > 0): the
                               narrowphase then takes the gap between the cores, dist - (core_a +
                               core_b), and the coating compression (_manager_process.py:351-360);
                               the broadphase keeps the outer radii */
} xk_mesh;

/* Pair table: _ContactPairOutput / _ContactStateOutput as structure of arrays
 * (xkep_cae/contact/_contact_pair.py:38-81).  Sorted by (ea, eb), ea < eb. */
typedef struct {
  int32_t n, cap;
  int32_t *ea, *eb;
  double *s, *t, *gap;
  double *normal, *t1, *t2; /* [3*cap] */
  double *lambda_n, *k_pen, *k_t, *p_n;
  double *z_t;              /* [2*cap] */
  double *q_trial_norm, *dissipation;
  uint8_t *status, *stick;  /* status: 0 INACTIVE, 1 ACTIVE, 2 SLIDING (_types.py:8-13) */
  /* Coating state (_contact_pair.py:57-62), NULL unless the mesh has core radii: coating_compression,
   * coating_compression_prev, coating_z_t [2*cap], coating_q_trial_norm, coating_dissipation,
   * coating_stick.  With coating every pair of the table is a member of the contact pattern, since
   * the reference evaluates the coating force of every pair. */
  double *coat_cc, *coat_cc_prev, *coat_z_t, *coat_qtn, *coat_diss;
  uint8_t* coat_stick;
} xk_pairs;

/* -------------------------------------------------------------- beam path */

/* Per-element reference frame [L0, R0 (3x3 row-major)] as 10 SoA columns of
 * n_elems doubles.  v_ref: host double[3] or NULL (smallest-component axis).
 * Replaces the reference-frame part of _assemble_cr_beam3d_batch_impl
 * (xkep_cae/elements/_beam_assembly.py:241-245, _beam_cr.py:831-853). */
xk_status xk_beam_reference(const xk_mesh* m, const double* v_ref, double* elem_ref, xk_stream s);

/* Colouring plan for a deterministic, atomic-free write of element blocks into
 * the fixed block-CSR pattern of K_T.  The element tangents are symmetrised
 * (_beam_assembly.py:322), so block (w, v) of K_T is the transpose of block
 * (v, w): the pattern holds the blocks with row <= column only, and each
 * element's off-diagonal block below the diagonal has block index -1 (not
 * written; the full K_T has the transpose of the stored block there). */
typedef struct {
  int32_t n_colors;
  const int32_t* color_ptr_host; /* host [n_colors+1], ranges of elem_order */
  const int32_t* elem_order;     /* [n_elems] elements grouped by colour */
  const int32_t* blk;            /* [4*n_elems] block index of (aa, ab, ba, bb) per element, -1 below the diagonal */
  const uint8_t* first;          /* [n_elems] bits 0..3: this element is the first writer of
                                    block aa, ab, ba, bb (aa / bb also: of the f rows of a / b) */
  int64_t nnzb;
  const int32_t* node_diag;      /* [n_nodes] or NULL: diagonal block of each node (-1: no element).
                                    Set only for chain meshes (every node in at most two elements,
                                    no two elements on the same two nodes); xk_beam_assemble32 then
                                    runs every element in one launch, adding the two contributions
                                    of a shared node (an order-free sum of two terms) */
  int32_t chain_ordered;         /* with node_diag: consecutive elements follow each other along every
                                    wire (element e's node b is element e+1's node a, or the node has
                                    one element); xk_beam_assemble32 then writes each shared node's
                                    sum once, without zeroing or atomics */
  int32_t beam_ctas_per_sm;      /* float kernel: 0 for one CTA per 128 threads of work, else at most
                                    this many CTAs per SM, looping (room for concurrent kernels) */
} xk_beam_plan;

/* Corotational Timoshenko internal force f_int and analytic tangent K_T of all
 * elements at displacement u: assemble_cr_beam3d (_beam_assembly.py:26-152)
 * as called by ULCRBeamAssembler.assemble_internal_force / assemble_tangent
 * (_beam_assembler.py:73-115).  f_int (double) and K_vals (double for XK_FP64,
 * float for XK_MIXED; 36*nnzb) may each be NULL.  Rows/blocks of nodes that
 * no element touches are not written. */
xk_status xk_beam_assemble(const xk_mesh* m, const xk_section* sec, const double* elem_ref,
                           const xk_beam_plan* plan, const double* u, int precision,
                           double* f_int, void* K_vals, xk_stream s);

/* Diagonal lumped mass (ULCRBeamAssembler.assemble_mass(lumped=True),
 * _beam_assembler.py:148-169, _beam_cr.py:267-296).  out: double[6*n_nodes],
 * overwritten. */
xk_status xk_beam_lumped_mass(const xk_mesh* m, const xk_section* sec, const xk_beam_plan* plan, double rho,
                              double* out, xk_stream s);

/* ------------------------------------------------------- strand meshes */

/* One layered helical strand of a mesh that may hold many (the batched
 * workload): the twisted-wire geometry of the reference's generator
 * (mesh/_twisted_wire.py:150-383, _make_twisted_wire_mesh at :271).  The
 * caller raises a non-negative gap to the generator's minimum safe gap first
 * (_twisted_wire.py:127-147,307-326). */
typedef struct {
  int32_t n_wires;          /* core + layers (3: three wires, no core) */
  int32_t n_elems_per_wire;
  int32_t lay_direction;    /* +1 / -1: twist of layer 1 */
  int32_t pad;
  double wire_diameter, pitch, length, gap;
  double x_offset;          /* shift along x of every node */
  int64_t node_first, elem_first; /* the strand's first node and element in the mesh */
} xk_strand_spec;

/* Node coordinates X (3 n_nodes), connectivity conn (2 n_elems), the layer of
 * every element (nullable) and the radii (nullable) of n_specs strands whose
 * specs (device memory, sorted by node_first and by elem_first) tile
 * [0, n_nodes) and [0, n_elems).  Elements run wire by wire, node i to i+1. */
xk_status xk_strand_generate(const xk_strand_spec* specs, int32_t n_specs, int64_t n_nodes, int64_t n_elems,
                             double* X, int32_t* conn, int32_t* elem_layer, double* radii, xk_stream s);

/* ----------------------------------------------------------- contact path */

typedef struct {
  double k_pen;            /* penalty (PenaltyStrategy.compute_k_pen) */
  double k_t_ratio;        /* tangential / normal penalty (_ContactConfigInput.k_t_ratio) */
  double mu_eff;           /* friction coefficient after the mu ramp (law_friction.py:183-195) */
  double smoothing_delta;  /* Huber smoothing; 0 = plain max(0, x) (contact_force/strategy.py:139) */
  double g_on, g_off;      /* active-set hysteresis (_manager_process.py:475-494) */
  int32_t allow_deactivation;
  /* Kelvin-Voigt coating (KelvinVoigtCoatingProcess, contact/coating/strategy.py:80-376), used when the
   * mesh has core radii: stiffness k, damping c, coating friction coefficient and tangential ratio, and
   * the step's pseudo-time increment for the dashpot (c > 0 and dt > 0). */
  double coat_k, coat_c, coat_mu, coat_kt_ratio, coat_dt;
} xk_contact_params;

typedef struct {
  double margin;                 /* AABB inflation added to every radius */
  int32_t exclude_shared;        /* drop pairs whose elements share a node */
  int32_t exclude_same_layer;    /* drop pairs of one layer (needs mesh layer) */
  int32_t midpoint_prescreening; /* _manager_process.py:260-286 */
  double prescreening_margin;    /* <= 0: half the mean of r_a + r_b over the candidates */
  double cell_size;              /* grid cell edge; <= 0: automatic.  Sets the work, never the result
                                    (the reference's cell_size, contact/_broadphase.py:18,55-58) */
} xk_bp_params;

/* Broadphase on the deformed coordinates X + u: every element pair (i<j) whose
 * closed inflated AABBs overlap, then the shared-node, same-layer and midpoint
 * filters; output sorted by (i, j).  Replaces _broadphase_aabb
 * (xkep_cae/contact/_broadphase.py:13-96) and the filtering part of
 * DetectCandidatesProcess.process (_manager_process.py:172-217).
 * out_pairs: int32[2*cap] as (i, j) rows.  If cap is too small the function
 * returns XK_ERR_CAPACITY and *n_out holds the required count.  n_raw and
 * n_prefilter (host, nullable) receive the raw AABB-overlap count and the count
 * before the midpoint prescreen.  Synchronises the stream. */
xk_status xk_broadphase(const xk_mesh* m, const double* u, const xk_bp_params* bp, int32_t* out_pairs,
                        int64_t cap, int64_t* n_out, int64_t* n_raw, int64_t* n_prefilter,
                        xk_stream s);

/* Pair-list update of DetectCandidatesProcess (_manager_process.py:219-250):
 * the union of `old` and the sorted candidates; old pairs that are not
 * candidates become INACTIVE with their state kept, new ones get a fresh state.
 * out->cap must be >= old->n + n_cands; out->n is set.  `old` may be empty. */
xk_status xk_pairs_merge(const xk_mesh* m, const xk_pairs* old, const int32_t* cands, int64_t n_cands,
                         xk_pairs* out, xk_stream s);

/* Narrowphase of every pair at X + u in exact reference arithmetic: closest
 * point, gap, transported frame (UpdateGeometryProcess.process,
 * _manager_process.py:327-403, geometry/_compute.py:55-261); with
 * update_active != 0 the active-set hysteresis follows
 * (_update_active_set_state, _manager_process.py:475-494). */
xk_status xk_narrowphase(const xk_mesh* m, xk_pairs* p, const double* u, const xk_contact_params* cp,
                         int update_active, xk_stream s);

/* The detection narrowphase of the mixed engine: UpdateGeometryProcess with
 * the active-set update (_manager_process.py:327-403, 475-494), every pair
 * first in float from node32 (xk_nodes_prepare at this u), and in exact
 * reference arithmetic (as xk_narrowphase) every pair whose float gap lies
 * within a bound of its error from [g_on, g_off], or that is near-parallel,
 * or on coated wires.  The status of every pair is the exact one; the stored
 * s, t, gap and frame of the others carry float rounding.  *n_exact (device,
 * nullable): how many pairs took the exact routine. */
xk_status xk_narrowphase_screened(const xk_mesh* m, xk_pairs* p, const double* u, const float* node32,
                                  const xk_contact_params* cp, int32_t* n_exact, xk_stream s);

#define XK_STAGE_NARROW 1   /* frozen-active-set narrowphase (_newton_steps.py:91-94) */
#define XK_STAGE_NORMAL 2   /* HuberContactForceProcess.evaluate (contact_force/strategy.py:126-170) */
#define XK_STAGE_FRICTION 4 /* CoulombReturnMappingProcess.evaluate (friction/strategy.py:111-148) */
#define XK_STAGE_TANGENT 8  /* .tangent of both (contact_force/strategy.py:172-254, friction/_assembly.py:108-257) */
#define XK_STAGE_NO_OTHERS 16  /* skip the other pairs' narrowphase (run it in another launch / stream) */
#define XK_STAGE_NO_MEMBERS 32 /* skip the member kernel (only the other pairs' narrowphase) */
#define XK_OUT_COMBINED 0   /* record (B = B_n - B_f, s, t, v = v_n + v_f): 14 values */
#define XK_OUT_SPLIT 1      /* record (s, t, v_n, v_f, B_n, B_f): 26 values */
/* Columns of a combined record: B first so that B, s and t are the first
 * twelve values (three 16-byte loads for float records). */
#define XK_REC_B 0
#define XK_REC_S 9          /* s, then t */
#define XK_REC_V 11
#define XK_REC_STRIDE_COMBINED 16 /* values per record in memory (padded) */
#define XK_REC_STRIDE_SPLIT 32

/* The pairs that can contribute in an increment ("members": status != INACTIVE
 * or p_n > 0 after detection and the active-set update), the rest, the node
 * incidence of the members and the block pattern of K_c with each block's
 * contributor list.  Built once per increment; every array is caller-owned.
 *
 * Block storage of K_c: a member adds c_k c_l B to block (node_k, node_l) and
 * the same c_l c_k B to block (node_l, node_k), so the block at (w, v) always
 * equals the block at (v, w) (the same 3x3 values, not the transpose).  The
 * pattern, and every K_c written by the gathers, hold the blocks with
 * row <= column only, in (row, column) order; the full matrix has the mirror
 * of every off-diagonal stored block as well (nnzb_full blocks in all). */
typedef struct {
  int32_t n_nodes;
  int32_t n_members, n_others;
  int64_t nnzb;        /* stored contact blocks (row <= column) */
  int64_t n_contrib;   /* contributions to the stored blocks (set by the build) */
  int64_t cap_members, cap_others, cap_blocks;
  int32_t* members;      /* [cap_members] pair index of each member, ascending */
  int32_t* member_nodes; /* [4*cap_members] nodes A0 A1 B0 B1 of each member */
  int32_t* others;       /* [cap_others] the remaining pairs, ascending */
  int32_t* inc_ptr;      /* [n_nodes+1] */
  int32_t* inc;          /* [4*cap_members] (member << 2) | local node k */
  int32_t* row_ptr;      /* [n_nodes+1] block rows of K_c */
  int32_t* col;          /* [cap_blocks] */
  int32_t* blk_row;      /* [cap_blocks] */
  int32_t* blk_ptr;      /* [cap_blocks+1] */
  int32_t* contrib;      /* [16*cap_members] (member << 4) | (k << 2) | l */
  /* Element-side form of the same sums (gather variant XK_GATHER_SIDES); built
   * when node_elem_ptr, node_elem, elem_ptr, elem_inc and bcodes are non-NULL.
   * A block's same-side contributions (k, l on one element) are sums over that
   * element's members, S_e^pq = sum c_p c_q B (p, q in {0,1}; three distinct
   * per element, 48 values with padding); each block lists at most four terms inline:
   * -1 empty, other negative values (offset | 0x80000000) an element sum at
   * elem_sums[offset], non-negative values a cross code (member << 4) |
   * (k << 2) | l.  Sorted ascending per block, so every sum has a fixed order. */
  int64_t n_elems;        /* set by the build */
  int64_t sides_ok;       /* set by the build: 1 if every block fits four terms (always for wire meshes) */
  int32_t* node_elem_ptr; /* [n_nodes+1] */
  int32_t* node_elem;     /* [4*n_elems] pairs ((element << 1) | local index, other node) */
  int32_t* elem_ptr;      /* [n_elems+1] */
  int32_t* elem_inc;      /* [2*cap_members] (member << 1) | side (0 = A, 1 = B) */
  int32_t* bcodes;        /* [4*cap_blocks] */
  void* elem_sums;        /* [56*n_elems] scratch of the record type: S^00, S^01, S^11 per element, each
                           * as 16 values (the 9 of the sum, then 1, 1 and padding); then, with
                           * combined records, the element force sums F^0, F^1 (8 values per element) */
  double* norm_scratch;   /* [(6*n_nodes + 255)/256 + 1] zero-initialised scratch of
                           * xk_contact_gather_force_elem's fused norm (block sums and a counter
                           * that each launch leaves at zero) */
  /* Lower index (built when both are non-NULL): for node w, low_blk[low_ptr[w] ..
   * low_ptr[w+1]) are the stored blocks (v, w) with v < w, ascending in v; the
   * full row w of K_c is those blocks' mirrors followed by the stored row. */
  int64_t nnzb_full;      /* set by the build: blocks of the full matrix (nnzb without the index) */
  int32_t* low_ptr;       /* [n_nodes+1] */
  int32_t* low_blk;       /* [cap_blocks] */
  /* Launch shape (0 = the built-in default): persistent CTAs per SM of the element-side block
   * gather (XK_GATHER_SIDES).  Results do not depend on it; an autotuner may choose it. */
  int32_t sides_per_sm;
  int32_t node_elem_ready; /* 1: node_elem_ptr / node_elem already hold the mesh's node -> element lists
                            * (set by the build; reset it to 0 when the mesh or those arrays change) */
} xk_contact_pattern;

/* Returns XK_ERR_CAPACITY (with n_members, n_others, nnzb set) when a capacity
 * is too small.  Synchronises the stream. */
xk_status xk_contact_pattern_build(const xk_mesh* m, const xk_pairs* p, xk_contact_pattern* pat,
                                   xk_stream s);

/* Per-iteration pair evaluation, fused over the selected stages.  A member's
 * translational force on its local node k (A0, A1, B0, B1) is c_k v and its
 * tangent block (k, l) is c_k c_l B with c = [1-s, s, -(1-t), -t]; these go
 * to the member's record rec[member*stride + value] (stride 16 for combined,
 * 32 for split records; double for XK_FP64, float for XK_MIXED; rec holds
 * stride*cap_members values).  With XK_STAGE_NARROW the other pairs get the
 * narrowphase too, as in the reference.  The four stages together replace the
 * contact part of ContactForceAssemblyProcess + TangentAssemblyProcess
 * (_newton_steps.py:79-135,289-313). */
xk_status xk_pair_step(const xk_mesh* m, xk_pairs* p, const xk_contact_pattern* pat, const double* u,
                       const double* u_ref, const xk_contact_params* cp, int stages, int precision,
                       int out_mode, void* rec, xk_stream s);

#define XK_WHICH_COMBINED 0
#define XK_WHICH_NORMAL 1
#define XK_WHICH_FRICTION 2

/* out[dof] = base[dof] + scale * sum_{members at the node} c_k v  - f_ext[dof],
 * then out[dof] = 0 where fixed[dof] != 0; base, f_ext, fixed nullable.  With
 * base = f_int and scale = -1 this is the residual R = f_int + f_c - f_ext of
 * ContactForceAssemblyProcess (_newton_steps.py:123-129); with base = NULL,
 * scale = 1 and which = normal / friction it is the force returned by
 * HuberContactForceProcess / CoulombReturnMappingProcess.evaluate.  norm2
 * (nullable, device double) receives sum(out^2) in a fixed-order FP64
 * reduction (ConvergenceCheckProcess, _newton_steps.py:194-203). */
xk_status xk_contact_gather_force(const xk_contact_pattern* pat, const void* rec, int precision, int out_mode,
                                  int which, const double* base, double scale, const double* f_ext,
                                  const uint8_t* fixed, double* out, double* norm2, xk_stream s);

/* K_c block values (9 per block, double|float, the nnzb stored blocks of the
 * pattern, row <= column; each off-diagonal one is also the block at the
 * mirrored position): sum over each block's contributors of c_k c_l B; which selects B_n - B_f (combined
 * records), B_n or B_f (split records).  variant picks the reduction schedule
 * (0 default, 1 one contributor per lane, 2 chunks of contributors per lane,
 * 3 element-side sums plus per-block cross lists, which needs the element-side
 * pattern and the elem_sums scratch; with combined records rec and elem_sums
 * must then be 32-byte aligned);
 * all give the same values for a given precision up to rounding order, each
 * deterministic. */
#define XK_GATHER_DEFAULT 0
#define XK_GATHER_LANES 1
#define XK_GATHER_CHUNKS 2
#define XK_GATHER_SIDES 3  /* element-side sums + cross lists (needs the element-side pattern) */
/* The two launches of XK_GATHER_SIDES as separate calls: the element sums (which also hold the
 * force sums that xk_contact_gather_force_elem reads), then the blocks from them.  A caller can
 * then start the residual while the blocks are gathered. */
#define XK_GATHER_SIDES_SUMS 4
#define XK_GATHER_SIDES_BLOCKS 5
xk_status xk_contact_gather_tangent(const xk_contact_pattern* pat, const void* rec, int precision, int out_mode,
                                    int which, int variant, void* Kc_vals, xk_stream s);

/* The residual of xk_contact_gather_force (out = base + scale * contact force
 * - f_ext, zero where fixed; norm2 nullable) from the element force sums that
 * the last element-side tangent gather (variant XK_GATHER_SIDES, combined
 * records) left in pat->elem_sums: each node
 * adds the sums of its incident elements, so the member records are not read
 * again.  Call it after that gather on the same stream (or after an event
 * recorded behind it).  The squared norm is fused: block sums in
 * pat->norm_scratch, added in block order by the last block, a fixed order.
 * Calls that overlap on one pattern race on norm_scratch. */
xk_status xk_contact_gather_force_elem(const xk_contact_pattern* pat, int precision, const double* base,
                                       double scale, const double* f_ext, const uint8_t* fixed, double* out,
                                       double* norm2, xk_stream s);

/* ------------------------------------------- mixed-precision fast path
 * The per-iteration kernels of the mixed path execute no double-precision
 * arithmetic: node positions are split once per iteration into float
 * high / low parts, the contact gap is taken in float-float arithmetic, the
 * beam frame in a cancellation-free float form, and the pair state lives in a
 * float copy of the table between increments. */
#define XK_NODE32_STRIDE 16 /* [x_hi(3), x_lo(3), u(6), u - u_ref(3), 0] per node */
#define XK_ELEM32_STRIDE 16 /* [X_b - X_a (3), L0, R0 (9), r_hi, r_lo, 0] per element */

/* Float copy of the pair state in slot order: the increment's members first
 * (slot = member index of the contact pattern), then the other pairs, so that
 * every per-iteration access is coalesced.  Node ids and the float-float
 * radius sum r_a + r_b are stored per slot. */
typedef struct {
  int32_t n, cap, n_members;
  int32_t* pair;           /* [cap] pair index of each slot */
  int32_t* nodes;          /* [4*cap] nodes A0 A1 B0 B1 */
  float* rad;              /* [2*cap] (hi, lo) of r_a + r_b */
  float *s, *t, *gap;
  float *normal, *t1, *t2; /* [3*cap] */
  float *p_n, *z_t;        /* z_t: [2*cap] */
  float *q_trial_norm, *dissipation, *k_pen, *k_t;
  uint8_t *status, *stick;
  float* mu;               /* [cap] friction coefficient of each slot, filled from xk_mesh.mu by xk_pairs_to32;
                              NULL (use xk_contact_params.mu_eff) unless the mesh has per-element mu */
  /* Coating (NULL unless the mesh has core radii): rad then holds the core radius sum; coat_total
   * (r_a - core_a) + (r_b - core_b) per slot and the coating state as in xk_pairs. */
  float *coat_total, *coat_cc, *coat_cc_prev, *coat_z_t, *coat_qtn, *coat_diss;
  uint8_t* coat_stick;
  int32_t* defer;          /* [2 * (cap + 2)] zero-initialised scratch or NULL: the pair kernels then
                              leave the rare near-parallel pairs to a second kernel each (other
                              pairs: [count, done, slots] from defer[0]; members: the same from
                              defer[cap + 2]), which keeps the exact double routine out of the common
                              kernels; each list is back at zero after its kernel */
  int32_t block;           /* threads per CTA of the other-pair and member kernels: a multiple of 32 up to
                              256, 0 = 256.  Results do not depend on it; an autotuner may choose it. */
  int32_t pad_launch;
  int32_t* slot;           /* [cap] or NULL: the slot of each pair of the FP64 table (the inverse of pair),
                              written by xk_pairs_to32, so that xk_pairs_from32 walks the table in its own
                              order (its writes coalesce) */
} xk_pairs32;

/* Per iteration: node records for the mixed kernels from u (and u_ref, nullable). */
xk_status xk_nodes_prepare(const xk_mesh* m, const double* u, const double* u_ref, float* node32, xk_stream s);

/* When the reference configuration changes: element records from xk_beam_reference's output. */
xk_status xk_beam_prepare32(const xk_mesh* m, const double* elem_ref, float* elem32, xk_stream s);

/* xk_beam_assemble in float from prepared records (f_int stays double). */
xk_status xk_beam_assemble32(const xk_mesh* m, const xk_section* sec, const float* elem32,
                             const xk_beam_plan* plan, const float* node32, double* f_int, float* K_vals,
                             xk_stream s);

/* Gather the pair table into the slot-ordered float copy (after the contact
 * pattern of the increment is built) and scatter it back (before the next
 * detection). */
xk_status xk_pairs_to32(const xk_mesh* m, const xk_pairs* p, const xk_contact_pattern* pat, xk_pairs32* q,
                        xk_stream s);
xk_status xk_pairs_from32(const xk_pairs32* q, xk_pairs* p, xk_stream s);

/* xk_pair_step with all four stages and combined float records on the float
 * state: slots [0, n_members) are the members (record index = slot), the rest
 * get the narrowphase only. */
#define XK_PAIRS_OTHERS 1  /* the narrowphase of the slots [n_members, n) */
#define XK_PAIRS_MEMBERS 2 /* the member kernel (narrowphase, normal, friction, tangent, records) */
#define XK_PAIRS_ALL 3
xk_status xk_pair_step32(xk_pairs32* q, const float* node32, const xk_contact_params* cp, float* rec, int parts,
                         xk_stream s);

/* Smooth (softplus) normal law for n gaps, element-wise:
 * _evaluate_smooth_normal_force_vectorized (contact/penalty/law_normal.py:129-149):
 * x = -g + lambda / k_pen, p_n = k_pen delta log(1 + exp(x / delta)),
 * dp_dg = -k_pen sigmoid(x / delta), with |x / delta| > 30 cut off as there.
 * lambdas may be NULL (all zero).  The reference's default law is the Huber
 * law of the pair kernels; this one is its C-infinity variant. */
xk_status xk_softplus_normal_law(int64_t n, const double* gaps, const double* lambdas, double k_pen, double delta,
                                 double* p_n, double* dp_dg, xk_stream s);

/* Constraint Jacobian rows c_k n of the non-INACTIVE pairs in table order
 * (_build_constraint_jacobian_ptp, xkep_cae/contact/geometry/strategy.py:83-132).
 * rows/cols/vals: [12*cap]; *n_rows (host) gets the number of active pairs;
 * XK_ERR_CAPACITY if cap < active pairs.  Synchronises the stream. */
xk_status xk_constraint_jacobian(const xk_mesh* m, const xk_pairs* p, int32_t* rows, int32_t* cols,
                                 double* vals, int32_t* pair_index, int64_t cap, int64_t* n_rows,
                                 xk_stream s);

/* ------------------------------------------------- coated-wire contact
 * KelvinVoigtCoatingProcess (contact/coating/strategy.py:80-400): a coating of
 * stiffness k and damping c between the wire cores, with Coulomb friction on
 * the coating surface.  Pair state of the coating, per pair of the table. */
typedef struct {
  double* cc;            /* [cap] coating_compression */
  double* cc_prev;       /* [cap] coating_compression_prev (the end of the previous step) */
  double* z_t;           /* [2*cap] coating_z_t, two planes */
  uint8_t* stick;        /* [cap] coating_stick */
  double* q_trial_norm;  /* [cap] coating_q_trial_norm */
  double* dissipation;   /* [cap] coating_dissipation */
} xk_coating_state;

typedef struct {
  double stiffness;  /* coating_stiffness k */
  double damping;    /* coating_damping c */
  double mu;         /* coating_mu */
  double k_t_ratio;  /* coating_k_t_ratio: tangential penalty k * ratio */
  double dt;         /* the step's pseudo-time increment (viscous term when c > 0 and dt > 0) */
} xk_coating_params;

/* The coating branch of UpdateGeometryProcess (_manager_process.py:351-360,
 * 386-396), after xk_narrowphase(update_active = 0) on a mesh whose radii are
 * the core radii (gap = dist - (core_a + core_b)): cc = max(0, coat_total -
 * gap) with coat_total[i] = (r_a - core_a) + (r_b - core_b); with
 * update_active, the active-set hysteresis with the coating term
 * (_update_active_set_state, :475-494: a compressed coating activates and
 * keeps a pair active). */
xk_status xk_coating_geometry(xk_pairs* p, const double* coat_total, const xk_contact_params* cp, int update_active,
                              double* cc, xk_stream s);

#define XK_COAT_FORCE 1            /* forces (strategy.py:97-143): v_n = -(k cc + c dcc/dt) n */
#define XK_COAT_TANGENT 2          /* stiffness (:145-196): B_n = (k + c / dt) n n^T where cc > 1e-15 */
#define XK_COAT_FRICTION 4         /* friction_forces (:198-288): return mapping, state update, v_f = -(q0 t1 + q1 t2) */
#define XK_COAT_FRICTION_TANGENT 8 /* friction_stiffness (:290-370): B_f = T D T^T from the coating friction state */
/* The selected coating stages over the members of pat (whose pair table
 * holds the geometry), as split records rec[member * 32 + value] (double):
 * s, t, v_n, v_f, B_n, B_f; gathered with xk_contact_gather_force /
 * xk_contact_gather_tangent, which = normal (elastic and viscous coating) or
 * friction.  u, u_ref (nullable): node-major displacements for the friction
 * slip. */
xk_status xk_coating_step(const xk_pairs* p, const xk_contact_pattern* pat, xk_coating_state* cs, const double* u,
                          const double* u_ref, const xk_coating_params* cp, int stages, double* rec, xk_stream s);

/* Gauss-point count of every pair for the line-to-line and mortar geometry
 * strategies with auto_gauss (_auto_select_n_gauss,
 * xkep_cae/contact/geometry/_compute.py:264-291, called from
 * LineToLineGaussProcess.update_geometry, geometry/strategy.py:436-451): from
 * the segment directions at X + u (u nullable: X), |cos| < 0.866 -> 2,
 * < 0.985 -> 3, else 5; default_n for a zero-length segment.  out: int8 [n]. */
xk_status xk_pair_gauss_points(const xk_mesh* m, const xk_pairs* p, const double* u, int32_t default_n,
                               int8_t* out, xk_stream s);

/* ------------------------------------------------------------------------
 * Generalized-alpha time integration with a lumped mass, no damping
 * (GeneralizedAlphaProcess, xkep_cae/time_integration/strategy.py:96-232);
 * alpha_m, alpha_f, gamma, beta from rho_inf as in :133-136.  All vectors are
 * device doubles of length n.
 * ---------------------------------------------------------------------- */
/* predict (:163-174): acc_old = acc, vel_old = vel,
 * u_pred = u + dt vel + 0.5 dt^2 (1 - 2 beta) acc, v_pred = vel + dt (1 - gamma) acc */
xk_status xk_genalpha_predict(int64_t n, const double* u, const double* vel, const double* acc,
                              double* vel_old, double* acc_old, double* u_pred, double* v_pred, double dt,
                              double beta, double gamma, xk_stream s);
/* correct (:176-185): acc = c0 (u - u_pred), vel = v_pred + dt gamma acc, c0 = 1 / (beta dt^2) */
xk_status xk_genalpha_correct(int64_t n, const double* u, const double* u_pred, const double* v_pred,
                              double* acc, double* vel, double dt, double beta, double gamma, xk_stream s);
/* effective_residual (:202-216): out = R + m ((1 - alpha_m) acc + alpha_m acc_old) */
xk_status xk_genalpha_residual(int64_t n, const double* R, const double* m, const double* acc,
                               const double* acc_old, double alpha_m, double* out, xk_stream s);
/* K[idx[i]] += c m[i] (K double for XK_FP64, float for XK_MIXED): the mass
 * term (1 - alpha_m) c0 M of effective_stiffness (:187-200) on the diagonal of
 * a block matrix, idx = value index of each DOF's diagonal entry (< 0: skipped). */
xk_status xk_add_diagonal(int64_t n, const int64_t* idx, const double* m, double c, int precision, void* K,
                          xk_stream s);

/* ------------------------------------------------------------------------
 * The Newton step's linear system on the device.  LinearSolveProcess
 * (xkep_cae/contact/solver/_newton_steps.py:338-366) solves K du = -R with the
 * rows and columns of the Dirichlet DOFs replaced by the identity, by a
 * sparse direct factorisation on the host.  Here K = K_beam + K_c stays in the
 * engine's block formats and is solved iteratively.
 * ---------------------------------------------------------------------- */
typedef struct {
  int32_t n_nodes;
  int32_t precision;            /* values double (XK_FP64) or float (XK_MIXED) */
  const int32_t* kb_row_ptr;    /* K_beam: its stored (row <= column) 6x6 blocks as block CSR [n_nodes+1] */
  const int32_t* kb_col;
  const void* kb_vals;          /* 36 per block, row-major */
  const int32_t* kb_blk_row;    /* row of every stored block, and per node w the stored blocks (v, w), */
  const int32_t* kb_low_ptr;    /*   v < w, ascending in v [n_nodes+1] / ...: their transposes complete */
  const int32_t* kb_low_blk;    /*   row w */
  const int32_t* kc_row_ptr;    /* K_c: the stored (row <= column) 3x3 blocks of xk_contact_pattern over */
  const int32_t* kc_col;        /*   the nodes' translational DOFs (nullable) */
  const void* kc_vals;          /* 9 per block */
  const int32_t* kc_blk_row;    /* the pattern's blk_row, low_ptr and low_blk: the mirrored blocks */
  const int32_t* kc_low_ptr;
  const int32_t* kc_low_blk;
  const uint8_t* fixed;         /* [6*n_nodes] Dirichlet DOFs (nullable): identity rows and columns */
} xk_system;

/* y = A x with A = K_beam + K_c (K_beam's stored blocks and their transposes, K_c's stored blocks
 * and their mirrors), Dirichlet rows and columns as the identity; x, y double [6*n_nodes]. */
xk_status xk_system_spmv(const xk_system* A, const double* x, double* y, xk_stream s);
/* dinv[36 v ...]: the inverse of every node's 6x6 diagonal block of A (the block-Jacobi preconditioner). */
xk_status xk_system_block_jacobi(const xk_system* A, double* dinv, xk_stream s);
/* BiCGStab with the block-Jacobi preconditioner dinv, from the initial x: until
 * ||b - A x|| <= rtol ||b|| (checked every check_every iterations) or max_iter.
 * work: double [8*6*n_nodes + 2*304 + 8].  The reductions are fixed-order, so
 * a solve is repeatable bit for bit; the iteration's scalars stay on the
 * device.  *iters and *rel_res (host, nullable) report the run. */
xk_status xk_bicgstab(const xk_system* A, const double* b, double* x, const double* dinv, double* work,
                      int32_t max_iter, int32_t check_every, double rtol, int32_t* iters, double* rel_res,
                      xk_stream s);
/* A (plus mass_coef * mass on the diagonal when mass is not null) as a dense
 * block-tridiagonal matrix for a direct factorisation: node v's DOF rows sit in
 * block row pos[v] / bn at local rows 6 (pos[v] % bn) + d; D, Lo, Up are nb
 * blocks of (6 bn)^2 doubles each (row-major), the diagonal blocks and the
 * blocks left and right of them.  Zeroes the three arrays first.  Couplings
 * more than one block row apart set *overflow (device int32) and are dropped:
 * choose bn at least the largest |pos[v] - pos[w]| of a stored block.  Padding
 * positions (n_nodes <= p < nb bn) are left zero for the caller. */
xk_status xk_system_blocktri(const xk_system* A, const int32_t* pos, int32_t bn, int32_t nb, const double* mass,
                             double mass_coef, double* D, double* Lo, double* Up, int32_t* overflow, xk_stream s);

/* ------------------------------------------------------------------------
 * Learned pruning of broadphase candidates.  No counterpart in the reference:
 * an MLP (XK_MLP_IN inputs -> 64 -> 64 -> 64 -> 1, ReLU, BF16 weights and
 * activations, FP32 accumulation) scores each candidate pair; candidates below
 * a threshold skip the pair table.  The exact broadphase + narrowphase stays
 * the referee (AssemblyEngine runs it every N detections).  Parameters are one
 * float vector of XK_MLP_PARAMS values: W1 (64 x 8), b1, W2 (64 x 64), b2,
 * W3 (64 x 64), b3, w4 (64), b4.
 * ---------------------------------------------------------------------- */
#define XK_MLP_IN 8
#define XK_MLP_HIDDEN 64
#define XK_MLP_PARAMS 8961
#define XK_MLP_ACT 192 /* a1, a2, a3 per sample */

/* Features of candidate pairs cands[2*i], cands[2*i+1] at the positions of
 * the node records node32 (xk_nodes_prepare: X + u as float hi/lo pairs):
 * midpoint separation, |cos| of the tangent angle, half lengths (all over
 * r_a + r_b), layer distance, core flag, previous-step gap (from `old`,
 * sorted by (ea, eb)) or, for a pair not in `old`, the current gap from the
 * clamped closest point in float, and whether the previous one exists.
 * feat: n x 8 float; hist[i] = 1 if the pair is in `old` with contact
 * history (status, p_n, k_pen or z_t set), such pairs are never pruned.
 * No counterpart in the reference (the learned pruning is this library's). */
xk_status xk_prune_features(const xk_mesh* m, const float* node32, const int32_t* cands, int64_t n,
                            const xk_pairs* old, float* feat, uint8_t* hist, xk_stream s);

/* Logits of n samples on the tensor cores (mma.sync BF16 -> FP32);
 * params_bf16: XK_MLP_PARAMS bfloat16 values. */
xk_status xk_mlp_forward(const uint16_t* params_bf16, const float* feat, int64_t n, float* logit, xk_stream s);

/* The same logits on the 5th-generation tensor cores: tcgen05.mma (BF16 ->
 * FP32) into a TMEM accumulator, 128 samples per tile, bias and ReLU applied
 * on the read-back.  params_bf16 and feat 16-byte aligned.  *err (device
 * int, caller-zeroed) is set to 1 if a tensor-core completion wait expired;
 * the logits are then undefined. */
xk_status xk_mlp_forward_tcgen05(const uint16_t* params_bf16, const float* feat, int64_t n, float* logit,
                                 int* err, xk_stream s);

/* Training: forward with stored activations (act: XK_MLP_ACT planes of n
 * floats), backward of the weighted mean binary cross-entropy (dvec: 192
 * planes of n; g: n; grad: XK_MLP_PARAMS, reduced in a fixed order; *loss on
 * the device), Adam (also writes the bf16 copy when theta_bf16 != NULL). */
xk_status xk_mlp_train_forward(const float* theta, const float* feat, int64_t n, float* act, float* logit,
                               xk_stream s);
xk_status xk_mlp_backward(const float* theta, const float* feat, const float* act, const float* logit,
                          const float* y, const float* w, int64_t n, float* dvec, float* g, float* grad,
                          float* loss, xk_stream s);
xk_status xk_mlp_adam(float* theta, const float* grad, float* m, float* v, int step, double lr, double beta1,
                      double beta2, double eps, uint16_t* theta_bf16, xk_stream s);
xk_status xk_mlp_to_bf16(const float* theta, uint16_t* out, xk_stream s);

/* Keep candidates with logit >= threshold or hist set (order kept), or with
 * invert != 0 the others (the pruned ones); *n_kept on the host.
 * score_error (device word, nullable): the error word of the tensor-core
 * scoring; when it is set the scores are undefined and every candidate is
 * kept.  *score_failed (host, nullable) receives that word.  Synchronises the
 * stream once.  No counterpart in the reference. */
xk_status xk_prune_select(const int32_t* cands, int64_t n, const float* logit, const uint8_t* hist,
                          float threshold, int invert, const int32_t* score_error, int32_t* kept,
                          int64_t* n_kept, int32_t* score_failed, xk_stream s);

/* Copy `in` to `out` without its pristine pairs (INACTIVE, p_n = k_pen = 0,
 * z_t = 0) that are not in the sorted list `kept`; order kept.  Synchronises
 * the stream. */
xk_status xk_pairs_drop_pristine(const xk_pairs* in, const int32_t* kept, int64_t n_kept, xk_pairs* out,
                                 xk_stream s);

/* xk_pairs_drop_pristine(old, cands) followed by xk_pairs_merge, in one merge: old pairs that are not
 * candidates stay (INACTIVE, state kept) only when they are not pristine.  The pair-list update of a
 * detection whose candidates were pruned.  Synchronises the stream. */
xk_status xk_pairs_merge_pruned(const xk_mesh* m, const xk_pairs* old, const int32_t* cands, int64_t n_cands,
                                xk_pairs* out, xk_stream s);

/* xk_constraint_jacobian without any device allocation, for callers that may
 * not allocate device memory while they run (a host whose device memory is all
 * handed to its own pool, a loop that must not go through the allocator).  No
 * counterpart in the reference: it is the same operation with the same
 * results; only where the scratch lives differs.
 *   - Scratch (a flag per pair, the scan's block sums, the active count) is a
 *     static 4 MiB device array in the library, so the pair table may hold at
 *     most XK_JACOBIAN_NOALLOC_MAX_PAIRS pairs; larger tables give XK_ERR_ARG
 *     (use xk_constraint_jacobian for them).
 *   - The first call in each context looks the array up (cudaGetSymbolAddress,
 *     with that device current); make that call before work that must not see
 *     a set-up step.  The address is kept per device together with the id of
 *     its context, so a new context on the device (after cudaDeviceReset, or a
 *     non-primary one) gets its own look-up.
 *   - The array is shared: calls on one device that overlap (two streams, two
 *     host threads) race on it and must be serialised by the caller.
 *   - Like xk_constraint_jacobian it synchronises the stream. */
#define XK_JACOBIAN_NOALLOC_MAX_PAIRS 1048576
xk_status xk_constraint_jacobian_noalloc(const xk_mesh* m, const xk_pairs* p, int32_t* rows, int32_t* cols,
                                         double* vals, int32_t* pair_index, int64_t cap, int64_t* n_rows,
                                         xk_stream s);

/* Fixed-order FP64 sum of squares of x[0..n) into *out (device). */
xk_status xk_norm2(const double* x, int64_t n, double* out, xk_stream s);

#ifdef __cplusplus
}
#endif

#endif /* XKGPU_H */
