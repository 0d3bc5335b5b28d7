"""Direct solve of the Newton system on the device, for strand meshes.

``LinearSolveProcess`` (``xkep_cae/contact/solver/_newton_steps.py:338-366``)
factorises ``K`` (Dirichlet rows and columns replaced by the identity) with a
sparse direct solver on the host.  The contact tangents of the strand states
are indefinite, which the device's iterative solve cannot handle
(``xkgpu.solve``), and the host's sparse LU fills badly on them (49 s for one
37-wire system).  A strand, though, is long and thin: numbering the nodes
along its axis, every element and every contact couples nodes a few
cross-sections apart.  ``BlockTridiagonalSolver`` therefore

1. orders the nodes along the axis of the mesh's largest extent (once per
   mesh) and takes the block size ``bn`` (nodes) as the largest distance in
   that order between two nodes of one stored block of K_beam or K_c (per
   contact pattern), so that ``K`` is block tridiagonal;
2. scatters ``K_beam + K_c`` (+ the time integrator's mass term) from the
   engine's block matrices into dense diagonal and off-diagonal blocks
   (``xk_system_blocktri``);
3. factorises with block LU, each diagonal block by an LU with partial
   pivoting on the device (cuSOLVER through ``torch.linalg``), in float32;
4. solves by GMRES in FP64 with that factorisation as the preconditioner, the
   system applied exactly by the engine's own SpMV.

The work is ``nb`` dense factorisations of size ``6 bn`` (37-wire strand:
about 620, 91-wire strand: about 1,500) and a few SpMVs per solve.
"""

from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np
import torch

from . import _lib as L
from .device import ptr, stream_handle
from .solve import DeviceLinearSolver


def blocktri_factor(D: torch.Tensor, Lo: torch.Tensor, Up: torch.Tensor) -> None:
    """Block LU of the block-tridiagonal matrix (diagonal blocks D, blocks left Lo, right Up; (nb, b, b)
    each), without pivoting between blocks: S_0 = D_0, S_i = D_i - Lo_i S_{i-1}^-1 Up_{i-1}.  D is
    overwritten by the inverses S_i^-1 (an LU with partial pivoting inside each block, on the device through
    ``torch.linalg``) and Up by S_i^-1 Up_i, so that applying the factors is matrix-vector products only.
    A singular S_i gives non-finite values downstream, as a singular sparse LU does."""
    nb = D.shape[0]
    for i in range(nb):
        if i > 0:
            D[i].sub_(Lo[i] @ Up[i - 1])
        inv, _ = torch.linalg.inv_ex(D[i])
        D[i].copy_(inv)
        if i < nb - 1:
            Up[i].copy_(inv @ Up[i])


def blocktri_apply(D: torch.Tensor, Lo: torch.Tensor, Up: torch.Tensor, rhs: torch.Tensor) -> torch.Tensor:
    """Solve with the factors of ``blocktri_factor`` for ``rhs`` (nb, b, k): y_i = S_i^-1 (r_i - Lo_i y_{i-1}),
    then y_i -= (S_i^-1 Up_i) y_{i+1} from the last block back."""
    nb = D.shape[0]
    rhs = rhs.to(D.dtype)
    y = torch.empty_like(rhs)
    for i in range(nb):
        r = rhs[i] if i == 0 else rhs[i] - Lo[i] @ y[i - 1]
        torch.matmul(D[i], r, out=y[i])
    for i in range(nb - 2, -1, -1):
        y[i] -= Up[i] @ y[i + 1]
    return y


def blocktri_solve(D: torch.Tensor, Lo: torch.Tensor, Up: torch.Tensor, rhs: torch.Tensor) -> torch.Tensor:
    """Factor (in place) and solve the block-tridiagonal system for ``rhs`` (nb, b, k)."""
    blocktri_factor(D, Lo, Up)
    return blocktri_apply(D, Lo, Up, rhs)


def gmres(matvec, b: torch.Tensor, precond, *, rtol: float = 1e-10, restart: int = 30, max_iter: int = 300):
    """Right-preconditioned restarted GMRES (Saad, Iterative Methods for Sparse Linear Systems, 2nd ed.,
    Alg. 9.5) in FP64, Gram-Schmidt repeated once, Givens rotations.  Stops at ``rtol`` or when a restart
    cycle no longer halves the residual (the attainable accuracy of an ill-conditioned system in FP64).
    Returns (x, iterations, relative residual)."""
    n = b.numel()
    bn = float(torch.linalg.vector_norm(b))
    x = torch.zeros_like(b)
    if bn == 0.0:
        return x, 0, 0.0
    it = 0
    rel = 1.0
    prev = math.inf
    while it < max_iter:
        r = b - matvec(x)
        beta = float(torch.linalg.vector_norm(r))
        rel = beta / bn
        if rel <= rtol or rel > 0.5 * prev:
            break
        prev = rel
        V = torch.zeros((restart + 1, n), dtype=b.dtype, device=b.device)
        Z = torch.zeros((restart, n), dtype=b.dtype, device=b.device)
        H = np.zeros((restart + 1, restart))
        cs, sn = np.zeros(restart), np.zeros(restart)
        g = np.zeros(restart + 1)
        g[0] = beta
        V[0] = r / beta
        k = 0
        while k < restart and it < max_iter:
            Z[k] = precond(V[k])
            w = matvec(Z[k])
            h = (V[: k + 1] @ w)  # classical Gram-Schmidt, repeated once for stability
            w = w - h @ V[: k + 1]
            h2 = V[: k + 1] @ w
            w = w - h2 @ V[: k + 1]
            hk = (h + h2).cpu().numpy()
            hn = float(torch.linalg.vector_norm(w))
            H[: k + 1, k] = hk
            H[k + 1, k] = hn
            for q in range(k):
                t = cs[q] * H[q, k] + sn[q] * H[q + 1, k]
                H[q + 1, k] = -sn[q] * H[q, k] + cs[q] * H[q + 1, k]
                H[q, k] = t
            den = float(np.hypot(H[k, k], H[k + 1, k]))
            cs[k], sn[k] = (H[k, k] / den, H[k + 1, k] / den) if den > 0.0 else (1.0, 0.0)
            H[k, k] = cs[k] * H[k, k] + sn[k] * H[k + 1, k]
            H[k + 1, k] = 0.0
            g[k + 1] = -sn[k] * g[k]
            g[k] = cs[k] * g[k]
            k += 1
            it += 1
            rel = abs(g[k]) / bn
            if hn > 0.0:
                V[k] = w / hn
            if rel <= rtol or hn == 0.0:
                break
        y = np.linalg.solve(np.triu(H[:k, :k]), g[:k]) if k else np.zeros(0)
        x = x + torch.as_tensor(y, dtype=b.dtype, device=b.device) @ Z[:k]
        if rel <= rtol:
            r = b - matvec(x)
            rel = float(torch.linalg.vector_norm(r)) / bn
            if rel <= rtol:
                break
    return x, it, rel


class BlockTridiagonalSolver:
    """``K du = -R`` for ``ContactFrictionSolver``: GMRES in FP64 on the device, preconditioned by the block
    LU of the axially ordered system.

    The factorisation runs in ``factor_dtype`` (float32 by default: the dense block products are ~60x
    faster than in FP64 on this GPU, and the FP32 factors are a near-exact preconditioner); the Krylov
    iteration applies the system itself in FP64 (``xk_system_spmv`` plus the mass term) until the
    relative residual is below ``rtol``.  With ``factor_dtype=torch.float64`` the preconditioned system
    is the identity up to the rounding of the block LU, which has no pivoting between blocks.

    The factors are kept across solves (Newton iterations, increments, contact patterns of the same block
    layout) while they stay a good preconditioner: a solve that needed more than ``refactor_iters`` Krylov
    iterations marks them for a new factorisation at the next solve, and a solve that does not reach the
    tolerance with kept factors factors the current system at once and solves again.  Since the Krylov
    iteration applies the exact system, the solution's accuracy does not depend on the factors' age.
    """

    def __init__(self, engine, axis: int | None = None, *, factor_dtype=torch.float32, rtol: float = 1e-10,
                 restart: int = 30, max_iter: int = 300, refactor_iters: int = 30):
        self.eng = engine
        dev = engine.device
        X = engine.mesh.X.reshape(-1, 3).cpu().numpy()
        if axis is None:
            axis = int(np.argmax(X.max(0) - X.min(0))) if len(X) else 2
        order = np.lexsort((np.arange(len(X)), X[:, axis]))  # along the axis, ties by node id
        pos = np.empty(len(X), dtype=np.int32)
        pos[order] = np.arange(len(X), dtype=np.int32)
        self.pos = torch.as_tensor(pos, device=dev)
        self.perm = (6 * self.pos.to(torch.int64)[:, None] + torch.arange(6, device=dev)).reshape(-1)
        self.n = len(X)
        self.factor_dtype = factor_dtype
        self.rtol, self.restart, self.max_iter = float(rtol), int(restart), int(max_iter)
        self.refactor_iters = int(refactor_iters)
        self._F = None  # the factors in use (fp32 copies or the FP64 blocks)
        self._need_factor = True
        self._graphs = {}  # the apply of each factor buffer set, captured as a CUDA graph
        self._sysw = DeviceLinearSolver(engine)  # the xk_system view of the engine's matrices and its SpMV
        self.overflow = torch.zeros(1, dtype=torch.int32, device=dev)
        self.bn = 0
        self.nb = 0
        self._buf = None
        self._fbuf = None
        self._pattern_version = None
        self.stats = {"solves": 0, "factorizations": 0, "gmres_iterations": 0, "max_rel_residual": 0.0,
                      "not_converged": 0, "stale_refactor": 0, "fp64_refactor": 0, "factor_s": 0.0, "gmres_s": 0.0}

    def _bandwidth(self) -> int:
        e = self.eng
        pos = self.pos.to(torch.int64)
        bw = 0
        nbb = e.beam.nnzb
        if nbb > 0:
            r = e.beam.blk_row[:nbb].to(torch.int64)
            c = e.beam.col[:nbb].to(torch.int64)
            bw = int((pos[r] - pos[c]).abs().max())
        pat = e.pattern
        if pat.nnzb > 0:
            r = pat.blk_row[: pat.nnzb].to(torch.int64)
            c = pat.col[: pat.nnzb].to(torch.int64)
            bw = max(bw, int((pos[r] - pos[c]).abs().max()))
        return max(bw, 1)

    def _prepare(self):
        ver = getattr(self.eng.pattern, "version", None)
        if self._buf is not None and ver == self._pattern_version:
            return
        self._pattern_version = ver
        bn = min(self._bandwidth(), max(self.n, 1))
        nb = -(-self.n // bn)
        if self._buf is not None and (bn, nb) == (self.bn, self.nb):
            return  # same block layout: kept factors remain a valid preconditioner
        b = 6 * bn
        self._buf = self._fbuf = self._F = None
        self._graphs = {}
        torch.cuda.empty_cache()
        dev = self.eng.device
        need = nb * b * b * (3 * 8 + (3 * 4 if self.factor_dtype != torch.float64 else 0))
        if need > 0.5 * torch.cuda.mem_get_info(dev)[0]:
            # a coupling across much of the mesh (a state far from a strand's): no block layout fits
            self.bn, self.nb = 0, 0
            return
        self._buf = tuple(torch.empty((nb, b, b), dtype=torch.float64, device=dev) for _ in range(3))
        if self.factor_dtype != torch.float64:
            self._fbuf = tuple(torch.empty((nb, b, b), dtype=self.factor_dtype, device=dev) for _ in range(3))
        self.bn, self.nb = bn, nb
        self._need_factor = True

    def _factor(self, mass_diag, fp64: bool):
        """Scatter the current system into the dense blocks and factor it (in ``factor_dtype``, or FP64)."""
        torch.cuda.synchronize(self.eng.device)
        t0 = time.perf_counter()
        D, Lo, Up = self._buf
        nb, bn, b = self.nb, self.bn, 6 * self.bn
        sysc = self._sysw._sync()
        L.call("xk_system_blocktri", C.byref(sysc), ptr(self.pos), bn, nb,
               ptr(mass_diag) if mass_diag is not None else None, 1.0, ptr(D), ptr(Lo), ptr(Up), ptr(self.overflow),
               stream_handle(None))
        if int(self.overflow.item()):
            raise RuntimeError("block-tridiagonal solve: a coupling reaches beyond the neighbouring block")
        pad = nb * bn - self.n
        if pad:  # positions past the last node: identity rows
            idx = torch.arange(6 * (bn - pad), b, device=D.device)
            D[nb - 1, idx, idx] = 1.0
        if self._fbuf is not None and not fp64:
            for dst, src in zip(self._fbuf, (D, Lo, Up)):
                dst.copy_(src)
            F = self._fbuf
        else:
            F = self._buf
        blocktri_factor(*F)
        self._F = F
        self._need_factor = False
        self.stats["factorizations"] += 1
        torch.cuda.synchronize(self.eng.device)
        self.stats["factor_s"] += time.perf_counter() - t0

    def _apply_graph(self, F):
        """(graph, input, output): ``blocktri_apply`` over the factor buffers F captured once as a CUDA
        graph (its ~3 nb launches replayed together); valid while the buffers live, whatever they hold."""
        key = F[0].data_ptr()
        g = self._graphs.get(key)
        if g is None:
            x_in = torch.zeros((self.nb, 6 * self.bn, 1), dtype=F[0].dtype, device=F[0].device)
            side = torch.cuda.Stream(device=F[0].device)
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):
                blocktri_apply(*F, x_in)  # warm-up outside the capture
            torch.cuda.current_stream().wait_stream(side)
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph):
                y = blocktri_apply(*F, x_in)
            g = (graph, x_in, y)
            self._graphs[key] = g
        return g

    def __call__(self, backend, R: torch.Tensor, fixed: np.ndarray, mass_diag: torch.Tensor | None):
        self._sysw.set_fixed(fixed)
        self._prepare()
        if self._buf is None:  # the layout would not fit in device memory: a failed solve (cutback)
            self.stats["too_large"] = self.stats.get("too_large", 0) + 1
            return None
        nb, b = self.nb, 6 * self.bn
        fresh = self._need_factor or self._F is None
        if fresh:
            self._factor(mass_diag, fp64=False)
        perm = self.perm
        free = torch.as_tensor(~np.asarray(fixed, dtype=bool), device=R.device)
        zero = torch.zeros((), dtype=torch.float64, device=R.device)

        def matvec(x):
            y = self._sysw.matvec(x)
            if mass_diag is not None:
                y = y + torch.where(free, mass_diag * x, zero)
            return y

        def precond(v):
            graph, x_in, y = self._apply_graph(self._F)
            x_in.view(-1)[perm] = v.to(x_in.dtype)  # positions past the last node stay zero
            graph.replay()
            return y.reshape(-1)[perm].to(torch.float64)

        rhs = torch.where(free, -R.to(torch.float64), zero)
        st = self.stats
        enough = max(1e3 * self.rtol, 1e-7)
        # kept factors get a short budget of iterations before they are replaced
        t0 = time.perf_counter()
        du, it, rel = gmres(matvec, rhs, precond, rtol=self.rtol, restart=self.restart,
                            max_iter=self.max_iter if fresh else min(self.max_iter, 3 * self.refactor_iters))
        st["gmres_s"] += time.perf_counter() - t0
        it_last = it
        tries = [] if fresh else ["stale"]
        if self._fbuf is not None:
            tries.append("fp64")
        for kind in tries:
            if rel <= enough:
                break
            # kept factors no longer precondition this system (stale), or the float32 factors of the
            # current one are too coarse (fp64): factor again and solve again
            st[kind + "_refactor"] += 1
            self._factor(mass_diag, fp64=(kind == "fp64"))
            t0 = time.perf_counter()
            du2, it2, rel2 = gmres(matvec, rhs, precond, rtol=self.rtol, restart=self.restart,
                                   max_iter=self.max_iter)
            st["gmres_s"] += time.perf_counter() - t0
            it += it2
            it_last = it2
            if rel2 < rel:
                du, rel = du2, rel2
            if kind == "fp64":
                self._need_factor = True  # the next system starts from float32 factors again
        if it_last > self.refactor_iters:
            self._need_factor = True
        st["solves"] += 1
        st["gmres_iterations"] += it
        st["max_rel_residual"] = max(st["max_rel_residual"], rel)
        if not rel <= self.rtol:
            st["not_converged"] += 1
        return du
