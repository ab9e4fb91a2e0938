"""CPU restatement of the reference GCGE block algebraic multigrid solver
(numpy/scipy).

TEST INFRASTRUCTURE ONLY - the checker for the GPU library's BlockAMG.  See
``oracle/__init__.py``.

The reference's BlockAMG (src/ops_lin_sol.c:466-715) is a V-cycle over a
caller-supplied hierarchy (A_l, P_l) whose smoother at every level is the
reference's BlockPCG (src/ops_lin_sol.c:140-437) with that level's iteration
cap, rate and tolerance.  Multivectors are Fortran-ordered float64 arrays,
column ranges half-open as the reference's start[2]/end[2].  Sparse products
use scipy's CSR/CSC products (the reference's app_ccs scatter SpMM computes
the same sums, app/app_ccs.c:116-131, up to summation order).
"""
from __future__ import annotations

import numpy as np


class PCGState:
    """The fields of the reference's BlockPCGSolver that BlockAMG reads
    (src/ops_lin_sol.h:29-40): niter and residual of the last solve."""

    def __init__(self):
        self.niter = 0
        self.residual = -1.0


def block_pcg(matvec, b, x, max_iter, rate, tol, tol_type="abs", state=None, user_norms=None):
    """BlockPCG, src/ops_lin_sol.c:140-437: CG on every column of x (n x k, in
    place) for A x = b, columns leaving when their residual norm falls below
    rate times its initial value or tol times the column's norm (1 for "abs",
    |b| for "rel", |user_norms[i]| for "user", the values the caller leaves in
    dbl_ws, :186-191).  Returns the
    state with niter and residual as the reference fills them (:406-410): the
    last residual of the column first in the int_ws list of unconverged
    columns after the last iteration (that list is compacted in place, so
    when every column has left it still names the first column that entered
    the last iteration), or the first column's initial residual when no
    iteration ran."""
    st = state if state is not None else PCGState()
    k = b.shape[1]
    if tol_type == "rel":                                   # :172-185
        norm_b = np.sqrt(np.einsum("ij,ij->j", b, b))
    elif tol_type == "user":                                # :186-191
        norm_b = np.abs(np.asarray(user_norms, dtype=np.float64)[:k])
    else:                                                   # :192-197
        norm_b = np.ones(k)
    r = b - matvec(x)                                       # :201-221
    rho2 = np.einsum("ij,ij->j", r, r)
    init_res = np.sqrt(rho2)
    unconv = [0] * k                                        # int_ws, compacted in place
    num = 0
    rho2c = np.zeros(k)
    for i in range(k):                                      # :238-247
        if init_res[i] > tol * norm_b[i]:
            unconv[num] = i
            rho2c[num] = rho2[i]
            num += 1
    rho1c = np.zeros(k)
    last_res = np.zeros(k)
    p = np.zeros_like(x, order="F")
    niter = 0
    while niter < max_iter and num > 0:                     # :256
        cols = np.array(unconv[:num])
        beta = np.zeros(num) if niter == 0 else rho2c[:num] / rho1c[:num]
        p[:, cols] = r[:, cols] + beta[None, :] * p[:, cols]   # :272-281
        w = matvec(p[:, cols])                                 # :283-296
        ptw = np.einsum("ij,ij->j", p[:, cols], w)             # :306
        rho1c[:num] = rho2c[:num]                              # :325
        alpha = rho2c[:num] / ptw                              # :332
        x[:, cols] += alpha[None, :] * p[:, cols]              # :335-340
        r[:, cols] -= alpha[None, :] * w                       # :342-344
        rho2c[:num] = np.einsum("ij,ij->j", r[:, cols], r[:, cols])  # :351-355
        last_res[cols] = np.sqrt(rho2c[:num])                  # :375
        pre, num = num, 0
        for i in range(pre):                                   # :383-394
            c = unconv[i]
            if last_res[c] > rate * init_res[c] and last_res[c] > tol * norm_b[c]:
                unconv[num] = c
                rho1c[num] = rho1c[i]
                rho2c[num] = rho2c[i]
                num += 1
        niter += 1
    st.niter = niter                                           # :406-410
    st.residual = last_res[unconv[0]] if niter > 0 else init_res[0]
    return st


def block_amg(A_list, P_list, b, x, max_iter, rate, tol, tol_type="abs"):
    """BlockAMG, src/ops_lin_sol.c:643-685, with its V-cycle
    BlockAlgebraicMultiGrid (:466-642): up to max_iter[0] cycles, stopping
    once the residual field of the last smoothing solve at level 0 is below
    tol[0].  A_list: scipy sparse level matrices; P_list: scipy sparse P_l
    (n_l x n_{l+1}); x (n_0 x k) is updated in place.  Returns (residual,
    cycles run)."""
    L = len(A_list)
    coarsest = L - 1

    def cycle(level, bl, xl):
        A = A_list[level]
        st = block_pcg(lambda v: A @ v, bl, xl, max_iter[2 * level + 1], rate[level],
                       tol[level], tol_type)                   # pre-smoothing, :485-502
        if level < coarsest:
            res = bl - A @ xl                                  # :516-530
            cb = P_list[level].T @ res                         # restriction, :544-545
            cx = np.zeros_like(cb, order="F")                  # :563
            cycle(level + 1, np.asfortranarray(cb), cx)        # :570
            xl += P_list[level] @ cx                           # prolongation + update, :577-600
            st = block_pcg(lambda v: A @ v, bl, xl, max_iter[2 * level + 2], rate[level],
                           tol[level], tol_type)               # post-smoothing, :611-627
        return st.residual                                     # :637

    residual, cycles = -1.0, 0
    for _ in range(max_iter[0]):                               # :654-659
        residual = cycle(0, b, x)
        cycles += 1
        if residual < tol[0]:
            break
    return residual, cycles
