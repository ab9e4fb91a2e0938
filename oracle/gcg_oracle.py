"""CPU restatement of the reference GCGE GCG eigensolver (numpy/scipy).

TEST INFRASTRUCTURE ONLY - the checker for the GPU library and the CPU
baseline of the benchmark.  See ``oracle/__init__.py``.

Every routine follows one function of the reference and cites it.  State that
the reference keeps in file-static globals (src/ops_eig_sol_gcg.c:44-55) lives
on the ``GCGOracle`` instance.  Multivectors are Fortran-ordered float64 numpy
arrays (the reference's column-major ``LAPACKVEC``, app/app_lapack.h:17-20);
column ranges are half-open like the reference's ``start[2]/end[2]``.
The sparse operator is applied with scipy's CSR product, which computes the
same sums as the reference's CCS scatter SpMM (app/app_ccs.c:116-131) for a
symmetric matrix, up to summation order.

Dense LAPACK calls of the reference map to scipy:
  dsyevx (src/ops_eig_sol_gcg.c:1145-1150) -> scipy.linalg.eigh(driver="evx")
  dgemm/ddot/dgemv (app/app_lapack.c:64-183) -> numpy matmul
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

DBL_EPSILON = np.finfo(np.float64).eps


@dataclass
class GCGParams:
    """GCG tunables as set by GCGE_Setparameters (src/ops_eig_sol_gcg.c:1878-1913)
    on top of EigenSolverSetup_GCG's static defaults (:1573-1623)."""
    nev_init: int
    nev_max: int
    block_size: int
    tol: tuple = (1e300, 1e-8)
    num_iter_max: int = 500
    gap_min: float = 1e-5
    check_conv_max_num: int = 50
    orth_method: str = "mgs"      # InitializeX / ComputeW orthogonalisation: "mgs" or "bgs"
    orth_block_size: int = -1
    orth_max_reorth: int = 2
    orth_zero_tol: float = 2 * DBL_EPSILON
    reorth_tol: float = 50 * DBL_EPSILON          # src/ops_orth.c:404
    cg_max_iter: int = 30
    cg_rate: float = 1e-2
    cg_tol: float = 1e-14
    cg_tol_type: str = "abs"
    cg_auto_shift: int = 1
    cg_shift: float = 0.0
    cg_order: int = 1                             # compW_cg_order: 1 ComputeW, 2 ComputeW12
    compRR_tol: float = 2 * DBL_EPSILON


@dataclass
class GCGResult:
    eval: np.ndarray
    evec: np.ndarray
    nconv: int
    niter: int
    times: dict = field(default_factory=dict)
    marks: list = field(default_factory=list)  # wall clock at solve start and each loop top


class GCGOracle:
    """One GCG solve of A x = lambda B x (B None means B = I)."""

    def __init__(self, A, B, params: GCGParams):
        self.A = A.tocsr() if hasattr(A, "tocsr") else A
        self.B = None if B is None else (B.tocsr() if hasattr(B, "tocsr") else B)
        self.p = params
        self.n = self.A.shape[0]
        self.sigma = 0.0
        self.times = {k: 0.0 for k in ("initX", "checkconv", "compP", "compRR", "compRV",
                                       "compW", "linsol", "compX")}
        self.stats = {"spmm": 0, "pcg_iters": 0}

    # ------------------------------------------------------------------
    # OPS primitives (app_ccs / app_lapack / ops_multi_vec defaults)
    # ------------------------------------------------------------------
    def matdot(self, M, X):
        """MatDotMultiVec: app/app_ccs.c:50-139 (mat NULL -> copy, :134-137)."""
        self.stats["spmm"] += 1
        if M is None:
            return X.copy(order="F")
        return np.asfortranarray(M @ X)

    def mat_dot_shift(self, X):
        """MatDotMultiVecShift: y = A x + sigma (B x or x), src/ops_eig_sol_gcg.c:64-97."""
        Y = self.matdot(self.A, X)
        if self.sigma != 0.0:
            if self.B is None:
                Y += self.sigma * X
            else:
                Y += self.sigma * self.matdot(self.B, X)
        return Y

    # ------------------------------------------------------------------
    # Orthogonalisation: src/ops_orth.c
    # ------------------------------------------------------------------
    def _orth_self(self, x, start_x, end_x, B):
        """OrthSelf, src/ops_orth.c:45-118.  Returns the new end_x."""
        p = self.p
        if end_x <= start_x:
            return end_x
        k = start_x
        while k < end_x:
            Bxk = self.matdot(B, x[:, k:k + 1])
            r = x[:, k:end_x].T @ Bxk[:, 0]
            rk = math.sqrt(r[0]) if r[0] >= 0 else float("nan")
            if rk < p.orth_zero_tol:   # a NaN norm is kept, as in the reference
                # drop column k: move the last column into its place (:64-74)
                if k < end_x - 1:
                    x[:, k] = x[:, end_x - 1]
                end_x -= 1
                continue
            inv = 1.0 / rk
            x[:, k] *= inv
            if k < end_x - 1:
                coef = r[1:] * (-inv)
                x[:, k + 1:end_x] += np.outer(x[:, k], coef)
                for _ in range(1, p.orth_max_reorth - 1):   # (:93) empty for max_reorth=2
                    Bxk = self.matdot(B, x[:, k:k + 1])
                    coef = -(x[:, k + 1:end_x].T @ Bxk[:, 0])
                    x[:, k + 1:end_x] += np.outer(x[:, k], coef)
                    if np.max(np.abs(coef)) < p.reorth_tol:
                        break
            k += 1
        return end_x

    def mgs(self, x, start_x, end_x, B, block_size=None):
        """ModifiedGramSchmidt, src/ops_orth.c:203-394.  Returns the new end_x."""
        p = self.p
        if end_x <= start_x:
            return end_x
        # remove the X0 = x[:, :start_x] component from X1 (:235-269)
        if start_x > 0:
            for _ in range(1 + p.orth_max_reorth):
                BX1 = self.matdot(B, x[:, start_x:end_x])
                coef = -(x[:, :start_x].T @ BX1)
                x[:, start_x:end_x] += x[:, :start_x] @ coef
                if np.max(np.abs(coef)) < p.reorth_tol:
                    break
        bsz = p.orth_block_size if block_size is None else block_size
        init_start = start_x
        if bsz <= 0:
            bsz = max((end_x - init_start) // 2, 2)
        bsz = min(bsz, end_x - init_start)
        while bsz > 0:
            e1 = self._orth_self(x, init_start, init_start + bsz, B)
            init_end = e1
            length = bsz - (e1 - init_start)
            length = min(length, end_x - e1 - length)
            if length > 0:   # refill the dropped slots from the tail (:295-307)
                x[:, init_end:init_end + length] = x[:, end_x - length:end_x]
            end_x = end_x - (bsz - (init_end - init_start))
            if init_end < end_x and init_start < init_end:
                BX0 = None
                for idx in range(1 + p.orth_max_reorth):
                    if BX0 is None or B is None:
                        BX0 = self.matdot(B, x[:, init_start:init_end])
                    coef = -(BX0.T @ x[:, init_end:end_x])
                    x[:, init_end:end_x] += x[:, init_start:init_end] @ coef
                    if np.max(np.abs(coef)) < p.reorth_tol:
                        break
            init_start = init_end
            bsz = min(bsz, end_x - init_start)
        return end_x

    def _orth_self_evp(self, x, start_x, end_x, B):
        """OrthSelfEVP, src/ops_orth.c:122-201: G = X^T B X = V diag(w) V^T
        (ascending, dsyev), X <- X V diag(w^-1/2) with the eigenvalues whose
        magnitude is at most orth_zero_tol dropped; repeated until nothing is
        dropped and sum |w^-1/2| = k to reorth_tol."""
        p = self.p
        for _ in range(1 + p.orth_max_reorth):
            if end_x == start_x:
                return end_x
            X = x[:, start_x:end_x]
            N = end_x - start_x
            G = X.T @ self.matdot(B, X)
            w, V = np.linalg.eigh(0.5 * (G + G.T))
            lin_dep = 0
            for k in range(N):
                if abs(w[k]) > p.orth_zero_tol:
                    w[k] = 1.0 / np.sqrt(w[k])
                else:
                    lin_dep += 1
            Y = (X @ V[:, lin_dep:]) * w[lin_dep:]
            end_x -= lin_dep
            x[:, start_x:end_x] = Y
            if lin_dep == 0 and abs(np.sum(np.abs(w)) - N) < p.reorth_tol:
                break
        return end_x

    def _orth_binary(self, x, start_x, end_x, B, bsz, evp):
        """OrthBinary, src/ops_orth.c:416-518: leaves of at most bsz columns by
        OrthSelfEVP (evp) or OrthSelf; otherwise the first half, CGS of the
        second half against it, the second half, and the second half's last
        columns moved into the first half's dropped slots."""
        p = self.p
        ncols = end_x - start_x
        if ncols <= 0:
            return end_x
        if ncols <= bsz:
            if evp:
                return self._orth_self_evp(x, start_x, end_x, B)
            return self._orth_self(x, start_x, end_x, B)
        s0, mid = start_x, start_x + ncols // 2
        e0 = self._orth_binary(x, s0, mid, B, bsz, evp)
        s1, e1 = mid, end_x
        if e0 > s0:
            BX0 = self.matdot(B, x[:, s0:e0])   # kept from the first pass (:451-463)
            for _ in range(1 + p.orth_max_reorth):
                coef = BX0.T @ x[:, s1:e1]
                x[:, s1:e1] -= x[:, s0:e0] @ coef
                if np.max(np.abs(coef)) < p.reorth_tol:
                    break
        e1 = self._orth_binary(x, s1, e1, B, bsz, evp)
        gap = mid - e0
        new_end = e1 - gap
        ln = min(gap, e1 - s1)
        if ln > 0:
            x[:, e0:e0 + ln] = x[:, e1 - ln:e1].copy()
        return new_end

    def bgs(self, x, start_x, end_x, B):
        """BinaryGramSchmidt, src/ops_orth.c:519-623.  Returns the new end_x."""
        p = self.p
        if end_x <= start_x:
            return end_x
        if start_x > 0:   # against the prefix, checked every pass (:540-561)
            for _ in range(1 + p.orth_max_reorth):
                coef = x[:, :start_x].T @ self.matdot(B, x[:, start_x:end_x])
                x[:, start_x:end_x] -= x[:, :start_x] @ coef
                if np.max(np.abs(coef)) < p.reorth_tol:
                    break
        # leaf method and size (:575-591): blocks under 16 columns use OrthSelf
        # with leaves of 4 (or the given size); wider ones OrthSelfEVP with
        # leaves of at most a quarter of the block
        k = end_x - start_x
        bsz = p.orth_block_size
        if k < 16:
            bsz = 4 if bsz <= 0 else bsz
            evp = False
        else:
            bsz = k // 4 if (bsz <= 0 or bsz > k // 4) else bsz
            evp = True
        return self._orth_binary(x, start_x, end_x, B, bsz, evp)

    def orth(self, x, start_x, end_x, B):
        """MultiVecOrth with the method of InitializeX / ComputeW
        (src/ops_eig_sol_gcg.c:119-141, :650-668)."""
        if self.p.orth_method == "bgs":
            return self.bgs(x, start_x, end_x, B)
        return self.mgs(x, start_x, end_x, B)

    # ------------------------------------------------------------------
    # BlockPCG: src/ops_lin_sol.c:140-437
    # ------------------------------------------------------------------
    def block_pcg(self, b, x):
        """Solve (A + sigma B) x = b column-wise in place (x: n x k, b: n x k)."""
        p = self.p
        k = b.shape[1]
        if p.cg_tol_type == "rel":
            norm_b = np.sqrt(np.einsum("ij,ij->j", b, b))
        else:
            norm_b = np.ones(k)
        r = b - self.mat_dot_shift(x)
        rho2_full = np.einsum("ij,ij->j", r, r)
        init_res = np.sqrt(rho2_full)
        unconv = [i for i in range(k) if init_res[i] > p.cg_tol * norm_b[i]]
        rho2 = rho2_full[unconv].copy()
        rho1 = np.zeros_like(rho2)
        last_res = np.zeros(k)
        pv = np.zeros_like(x, order="F")
        niter = 0
        while niter < p.cg_max_iter and len(unconv) > 0:
            u = np.array(unconv)
            if niter == 0:
                pv[:, u] = r[:, u]
            else:
                pv[:, u] = r[:, u] + (rho2 / rho1)[None, :] * pv[:, u]
            w = self.mat_dot_shift(pv[:, u])
            pTw = np.einsum("ij,ij->j", pv[:, u], w)
            rho1 = rho2.copy()
            alpha = rho2 / pTw
            x[:, u] += alpha[None, :] * pv[:, u]
            r[:, u] -= alpha[None, :] * w
            rho2 = np.einsum("ij,ij->j", r[:, u], r[:, u])
            last_res[u] = np.sqrt(rho2)
            keep = [(i, c) for i, c in enumerate(unconv)
                    if last_res[c] > p.cg_rate * init_res[c] and last_res[c] > p.cg_tol * norm_b[c]]
            unconv = [c for _, c in keep]
            idx = [i for i, _ in keep]
            rho1 = rho1[idx]
            rho2 = rho2[idx]
            niter += 1
        self.stats["pcg_iters"] += niter
        return niter

    # ------------------------------------------------------------------
    # GCG phases: src/ops_eig_sol_gcg.c
    # ------------------------------------------------------------------
    def initialize_x(self, V, ritz_vec, nev_given):
        """InitializeX, :102-159."""
        V[:, :nev_given] = ritz_vec[:, :nev_given]
        nev_given = self.orth(V, 0, nev_given, self.B)
        if self.sizeX > nev_given:
            # libc rand() fill (app/app_lapack.c:322-333); not reached when
            # the caller supplies nevInit independent vectors
            rng = np.random.default_rng(0)
            V[:, nev_given:self.sizeX] = rng.random((self.n, self.sizeX - nev_given))
        self.endX = self.orth(V, nev_given, self.sizeX, self.B)
        assert self.endX == self.sizeX

    def compute_ritz_vec(self, ritz_vec, V):
        """ComputeRitzVec, :160-195: ritz_vec[startN:endX] = V[startN:endW] ss_evec."""
        s = self.sizeV - self.sizeC
        coef = self.ss_evec[:s, :self.endX - self.startN]
        ritz_vec[:, self.startN:self.endX] = V[:, self.startN:self.endW] @ coef

    def check_convergence(self, ritz_vec, num_check, offset):
        """CheckConvergence, :196-321.  Fills offset in place, returns nevConv."""
        tol = self.p.tol
        sN = self.startN
        X = ritz_vec[:, sN:sN + num_check]
        AX = self.matdot(self.A, X)
        BX = self.matdot(self.B, X)
        lam = self.ss_eval[sN:sN + num_check]
        R = AX - BX * lam[None, :]
        res = np.sqrt(np.einsum("ij,ij->j", R, R))
        self.last_residuals = res
        idx = 0
        while idx < num_check:
            if res[idx] > tol[0] or res[idx] > abs(lam[idx]) * tol[1]:
                break
            idx += 1
        while idx > 0:
            a, b = self.ss_eval[sN + idx - 1], self.ss_eval[sN + idx]
            if abs((a - b) / a) > self.p.gap_min:
                break
            idx -= 1
        nev_conv = self.sizeC + idx
        offset[0] = 0
        state = 1
        num_unconv = 0
        for i in range(num_check):
            if res[i] > tol[0] or res[i] > abs(lam[i]) * tol[1]:
                if state:
                    offset[offset[0] * 2 + 1] = sN + i
                    state = 0
                num_unconv += 1
                if num_unconv == self.sizeN:
                    offset[offset[0] * 2 + 2] = sN + i + 1
                    offset[0] += 1
                    break
            else:
                if not state:
                    offset[offset[0] * 2 + 2] = sN + i
                    offset[0] += 1
                    state = 1
        if num_unconv < self.sizeN:
            if state == 1:
                offset[offset[0] * 2 + 1] = sN + num_check
            e = sN + num_check + self.sizeN - num_unconv
            offset[offset[0] * 2 + 2] = min(e, self.endX)
            assert offset[offset[0] * 2 + 1] < offset[offset[0] * 2 + 2]
            offset[0] += 1
        assert offset[0] > 0
        return nev_conv

    def compute_p(self, V, offset):
        """ComputeP, :322-463 (small-space P coefficients, MGS in small space)."""
        s = self.sizeV - self.sizeC
        ev = self.ss_evec  # s x s (current layout)
        cols = []
        for i in range(offset[0]):
            o1, o2 = offset[2 * i + 1], offset[2 * i + 2]
            cols.extend(range(o1 - self.sizeC, o2 - self.sizeC))
        sizeP = len(cols)
        base = self.sizeX - self.sizeC
        work = np.zeros((s, base + sizeP), order="F")
        work[:, :base] = ev[:s, :base]
        work[:, base:] = ev[:s, cols]
        for i in range(offset[0]):
            o1, o2 = offset[2 * i + 1], offset[2 * i + 2]
            work[o1 - self.sizeC:o2 - self.sizeC, base:] = 0.0
        # small-space MGS with B = NULL on the lapack backend (:385-419)
        endP_local = self.mgs(work, base, base + sizeP, None)
        self.ss_evec = np.zeros((s, s), order="F")
        self.ss_evec[:, :endP_local] = work[:, :endP_local]
        self.ss_evec[:, :base] = ev[:s, :base]
        self.startP = base + self.sizeC
        self.endP = endP_local + self.sizeC
        self.sizeP = self.endP - self.startP
        coef = self.ss_evec[:, base:endP_local]
        P = V[:, self.startN:self.endW] @ coef
        V[:, self.startP:self.endP] = P

    def compute_x(self, V, ritz_vec):
        """ComputeX, :464-477."""
        V[:, self.startN:self.endX] = ritz_vec[:, self.startN:self.endX]

    def compute_w(self, V, ritz_vec, offset):
        """ComputeW (compW_cg_order 1), :478-701."""
        p = self.p
        sigma = 0.0
        if p.cg_auto_shift == 1:
            sc = self.sizeC
            sigma = -self.ss_eval[sc] + (self.ss_eval[sc + 1] - self.ss_eval[sc]) * 0.01
        self.sigma = p.cg_shift + sigma
        self.startW = self.endP
        bsz = 0
        bcols = []
        for i in range(offset[0]):
            o1, o2 = offset[2 * i + 1], offset[2 * i + 2]
            ln = o2 - o1
            V[:, self.startW + bsz:self.startW + bsz + ln] = ritz_vec[:, o1:o2]
            bb = self.matdot(self.B, V[:, o1:o2]) * (self.ss_eval[o1:o2] + self.sigma)[None, :]
            bcols.append(bb)
            bsz += ln
        self.endW = self.startW + bsz
        b = np.asfortranarray(np.concatenate(bcols, axis=1))
        t0 = time.perf_counter()
        xw = np.asfortranarray(V[:, self.startW:self.endW])
        self.block_pcg(b, xw)
        V[:, self.startW:self.endW] = xw
        self.times["linsol"] += time.perf_counter() - t0
        # b aliases ritz_vec columns [offset[1], offset[1]+bsz) and is clobbered
        # there (:484, :527); ComputeRitzVec rewrites those columns later
        self.endW = self.orth(V, self.startW, self.endW, self.B)
        self.sizeW = self.endW - self.startW

    def compute_w12(self, V, ritz_vec, offset):
        """ComputeW12 (compW_cg_order 2), :703-929, on the branch app_ccs takes
        (no MatAxpby): the first total/2 unconverged columns (:757-790) get the
        BlockPCG solution x1 from their Ritz vectors (:807) and a second solve of
        the same system restarted from x1 (:815-901; the right-hand side is
        rebuilt there only because the shifted product used it as scratch)."""
        p = self.p
        sigma = 0.0
        if p.cg_auto_shift == 1:
            sc = self.sizeC
            sigma = -self.ss_eval[sc] + (self.ss_eval[sc + 1] - self.ss_eval[sc]) * 0.01
        self.sigma = p.cg_shift + sigma
        self.startW = self.endP
        total = sum(offset[2 * i + 2] - offset[2 * i + 1] for i in range(offset[0]))
        half = total // 2
        bsz = 0
        bcols = []
        for i in range(offset[0]):
            o1 = offset[2 * i + 1]
            ln = offset[2 * i + 2] - o1
            if bsz + ln >= half:
                ln = half - bsz
            V[:, self.startW + bsz:self.startW + bsz + ln] = ritz_vec[:, o1:o1 + ln]
            bcols.append(self.matdot(self.B, V[:, o1:o1 + ln])
                         * (self.ss_eval[o1:o1 + ln] + self.sigma)[None, :])
            bsz += ln
            if bsz >= half:
                break
        t0 = time.perf_counter()
        w0 = self.startW
        if bsz > 0:
            b = np.asfortranarray(np.concatenate(bcols, axis=1))
            for _ in range(2):
                xw = np.asfortranarray(V[:, w0:w0 + bsz])
                self.block_pcg(b, xw)
                V[:, w0:w0 + bsz] = xw
                if w0 == self.startW:      # x2 starts from x1 (:810-814)
                    V[:, w0 + bsz:w0 + 2 * bsz] = xw
                w0 += bsz
        self.times["linsol"] += time.perf_counter() - t0
        self.endW = self.startW + 2 * bsz
        self.endW = self.orth(V, self.startW, self.endW, self.B)
        self.sizeW = self.endW - self.startW

    def compute_rayleigh_ritz(self, V, nev_conv):
        """ComputeRayleighRitz, :931-1258."""
        p = self.p
        ptap = None
        if self.sizeP > 0:
            Pc = self.ss_evec[:, self.sizeX - self.sizeC:self.sizeX - self.sizeC + self.sizeP]
            ptap = Pc.T @ (self.ss_matA @ Pc)
        self.sizeV = self.sizeX + self.sizeP + self.sizeW
        self.startN += nev_conv - self.sizeC
        self.endN += nev_conv - self.sizeC
        self.endN = min(self.endN, self.endX)
        self.sizeN = self.endN - self.startN
        self.sizeC = nev_conv
        s = self.sizeV - self.sizeC
        M = np.zeros((s, s), order="F")
        xp = self.sizeX + self.sizeP - self.sizeC
        if self.sizeW > 0:
            AW = self.matdot(self.A, V[:, self.startW:self.endW])
            blk = V[:, self.startN:self.endW].T @ AW
            M[:, xp:] = blk
            M[xp:, :xp] = blk[:xp, :].T
        if self.sizeX == self.sizeV:
            bs = min(p.block_size, self.sizeX - self.sizeC)
            c0 = self.sizeC
            while c0 < self.sizeX:
                c1 = min(c0 + bs, self.sizeX)
                AV = self.matdot(self.A, V[:, c0:c1])
                M[:, c0 - self.sizeC:c1 - self.sizeC] = V[:, self.sizeC:self.sizeX].T @ AV
                c0 = c1
        else:
            M[:xp, :xp] = 0.0
            nx = self.sizeX - self.sizeC
            M[np.arange(nx), np.arange(nx)] = self.ss_eval[self.sizeC:self.sizeX]
            if ptap is not None:
                M[nx:nx + self.sizeP, nx:nx + self.sizeP] = ptap
        self.ss_matA = M.copy(order="F")
        Msh = M.copy()
        if p.cg_shift != 0.0:
            Msh[np.arange(s), np.arange(s)] += p.cg_shift
        import scipy.linalg as sla
        w, z = sla.eigh(Msh, lower=False, driver="evx")
        if p.cg_shift != 0.0:
            w = w - p.cg_shift
        self.ss_eval[self.sizeC:self.sizeC + s] = w
        self.ss_evec = np.asfortranarray(z)

    # ------------------------------------------------------------------
    # GCG outer loop: :1259-1562
    # ------------------------------------------------------------------
    def solve(self, evec0: np.ndarray, nev: int, nev_given: int | None = None) -> GCGResult:
        p = self.p
        n = self.n
        bs = p.block_size
        nev_init, nev_max = p.nev_init, p.nev_max
        if nev_given is None:
            nev_given = evec0.shape[1]
        assert nev_init >= nev_given and nev_init <= nev_max
        assert nev_init >= 3 * bs or nev_init == nev_max
        assert nev_max >= nev + bs or nev_max >= bs  # (:1283) with nevConv input = nev
        ritz_vec = np.zeros((n, nev_max), order="F")
        ritz_vec[:, :nev_given] = evec0[:, :nev_given]
        V = np.zeros((n, nev_max + 2 * bs), order="F")
        self.sizeC = 0
        self.sizeN = bs
        self.sizeX = nev_init
        self.sizeP = 0
        self.sizeW = 0
        self.sizeV = self.sizeX
        self.startN = 0
        self.endN = self.startN + self.sizeN
        self.endX = self.sizeX
        self.startP = self.endX
        self.endP = self.startP
        self.startW = self.endP
        self.endW = self.startW
        self.ss_eval = np.ones(nev_max + 2 * bs)
        self.ss_matA = None
        self.ss_evec = None
        offsetP = [0] * (bs + 3)
        offsetW = [0] * (bs + 3)
        marks = [time.perf_counter()]
        t = time.perf_counter()
        self.initialize_x(V, ritz_vec, nev_given)
        self.times["initX"] += time.perf_counter() - t
        t = time.perf_counter()
        self.compute_rayleigh_ritz(V, 0)
        self.times["compRR"] += time.perf_counter() - t
        self.ss_eval[self.sizeV:] = self.ss_eval[self.sizeV - 1]
        t = time.perf_counter()
        self.compute_ritz_vec(ritz_vec, V)
        self.times["compRV"] += time.perf_counter() - t
        nev0 = min(nev, nev_max)
        nevc = 0
        nev_target = 2 * bs if nev_init < nev_max else nev0
        nev_target = min(nev_target, nev0)
        num_iter_max = p.num_iter_max
        num_iter = 0
        while True:
            marks.append(time.perf_counter())
            num_check = 0 if num_iter <= 0 else (
                self.sizeN if self.startN + self.sizeN < self.endX else self.endX - self.startN)
            num_check = min(num_check, p.check_conv_max_num)
            if num_check == 0:
                num_check = 1
            t = time.perf_counter()
            nevc = self.check_convergence(ritz_vec, num_check, offsetW)
            self.times["checkconv"] += time.perf_counter() - t
            if nevc >= nev_target:
                if nevc >= nev0:
                    break
                nev_target = min(nev_target + self.sizeP + self.sizeW, nev0)
                newX = min(self.sizeX + self.sizeP + self.sizeW, nev_max)
                s = self.sizeV - self.sizeC
                coef = self.ss_evec[:s, self.endX - self.sizeC:newX - self.sizeC]
                ritz_vec[:, self.endX:newX] = V[:, self.startN:self.endW] @ coef
                self.sizeX = newX
                self.sizeP = 0
                self.sizeW = 0
                self.sizeV = self.sizeX
                self.startP = self.endX
                self.endP = self.startP
                self.startW = self.endP
                self.endW = self.startW
                self.endX = self.sizeX
                self.endN = min(self.startN + bs, self.endX)
                self.sizeN = self.endN - self.startN
                num_iter_max -= num_iter
                num_iter = 0
            t = time.perf_counter()
            if num_iter == 0:
                self.sizeP = 0
                self.startP = self.endX
                self.endP = self.startP
            else:
                self.compute_p(V, offsetP)
            self.times["compP"] += time.perf_counter() - t
            t = time.perf_counter()
            self.compute_x(V, ritz_vec)
            self.times["compX"] += time.perf_counter() - t
            t = time.perf_counter()
            if self.p.cg_order != 1:   # (:1456-1461)
                self.compute_w12(V, ritz_vec, offsetW)
            else:
                self.compute_w(V, ritz_vec, offsetW)
            self.times["compW"] += time.perf_counter() - t
            offsetP, offsetW = offsetW, offsetP
            t = time.perf_counter()
            self.compute_rayleigh_ritz(V, nevc)
            self.times["compRR"] += time.perf_counter() - t
            self.ss_eval[self.sizeV:] = self.ss_eval[self.sizeV - 1]
            t = time.perf_counter()
            self.compute_ritz_vec(ritz_vec, V)
            self.times["compRV"] += time.perf_counter() - t
            num_iter += 1
            if num_iter >= num_iter_max:
                break
        niter = num_iter + (p.num_iter_max - num_iter_max)
        ev = np.zeros(nev_max)
        ev[:self.sizeX] = self.ss_eval[:self.sizeX]
        marks.append(time.perf_counter())
        return GCGResult(eval=ev, evec=ritz_vec, nconv=nevc, niter=niter, times=dict(self.times),
                         marks=marks)


def gcg_solve(A, B, X0, nev, block_size, nev_init, nev_max, tol=(1e300, 1e-8),
              max_iter=500, gap_min=1e-5, auto_shift=1, orth=None, w_order=1) -> GCGResult:
    """Convenience wrapper: the reference's default GCGE parameter set;
    orth = (method, block_size) as EigenSolverSetParameters_GCG sets it for
    InitializeX and ComputeW; w_order = compW_cg_order."""
    p = GCGParams(nev_init=nev_init, nev_max=nev_max, block_size=block_size, tol=tuple(tol),
                  num_iter_max=max_iter, gap_min=gap_min, cg_auto_shift=auto_shift,
                  cg_order=w_order)
    if orth is not None:
        p.orth_method, p.orth_block_size = orth
    return GCGOracle(A, B, p).solve(np.asfortranarray(X0), nev)


def residuals(A, B, evals, evecs):
    """||A x - lambda B x||_2 and the same divided by |lambda|, per column."""
    AX = A @ evecs
    BX = evecs if B is None else B @ evecs
    R = AX - BX * evals[None, :]
    r = np.sqrt(np.einsum("ij,ij->j", R, R))
    return r, r / np.abs(evals)
