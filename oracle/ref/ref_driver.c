/*
 * Driver around the reference GCGE CPU path (app_ccs backend + GCG), compiled
 * together with the unmodified reference sources into oracle/_ref/.  Test
 * infrastructure only: used to generate the golden fixtures and as the
 * reference arm of the CPU baseline in this container.
 *
 * The call sequence is the one the reference's own front end uses
 * (gcge.c:490-517): OPS_Create, backend Set, OPS_Setup, MultiVecCreateByMat
 * for evec, GCGE_Create for the four multivector workspaces, dbl_ws/int_ws
 * sized as in gcge.c:503-510 (= src/ops_eig_sol_gcg.c:1647-1651),
 * EigenSolverSetup_GCG, GCGE_Setparameters, ops->EigenSolver.
 * The backend is app_ccs (app/app_ccs.c:213-249), the reference's sparse CCS
 * operator with int32 indices and FP64 values.  Besides GCG: one call of the
 * reference's MultiVecOrth (ref_orth) and of its BlockAMG (ref_block_amg).
 */
#include <stdlib.h>
#include <string.h>

#include "ops.h"
#include "app_ccs.h"
#include "ops_eig_sol_gcg.h"

/* As ref_gcg_solve, with the orthogonalisation method of InitializeX and
 * ComputeW chosen through the reference's own setter
 * (EigenSolverSetParameters_GCG, src/ops_eig_sol_gcg.c:1684-1741): orth_method
 * "mgs" or "bgs" (NULL: the GCGE_Setparameters default) and its block size;
 * then argv (argc entries, may be 0) through the reference's command-line
 * setter (EigenSolverSetParametersFromCommandLine_GCG, :1743-1862), e.g.
 * {"-gcge_compW_cg_order", "2"}. */
int ref_gcg_solve_opts(int n,
                  const int *a_colptr, const int *a_rowind, const double *a_val,
                  const int *b_colptr, const int *b_rowind, const double *b_val,
                  int nev, int block_size, int nev_init, int nev_max, int max_iter,
                  double abs_tol, double rel_tol, double gap_min, int auto_shift,
                  const double *x0, int nev_given,
                  double *eval_out, double *evec_out, int *nconv_out, int *niter_out,
                  const char *orth_method, int orth_block_size, int argc, char **argv)
{
    OPS *ops = NULL;
    OPS_Create(&ops);
    OPS_CCS_Set(ops);
    OPS_Setup(ops);

    CCSMAT A, B;
    A.data = (double *)a_val; A.i_row = (int *)a_rowind; A.j_col = (int *)a_colptr;
    A.nrows = n; A.ncols = n;
    void *matB = NULL;
    if (b_colptr != NULL) {
        B.data = (double *)b_val; B.i_row = (int *)b_rowind; B.j_col = (int *)b_colptr;
        B.nrows = n; B.ncols = n;
        matB = &B;
    }

    double *eval = calloc((size_t)nev_max, sizeof(double));
    void **evec = NULL;
    ops->MultiVecCreateByMat(&evec, nev_max, &A, ops);
    LAPACKVEC *ev = (LAPACKVEC *)evec;
    if (nev_given > 0)
        memcpy(ev->data, x0, sizeof(double) * (size_t)n * (size_t)nev_given);

    srand(0);
    void **mv_ws[4];
    GCGE_Create(&A, nev_max, block_size, nev_init, mv_ws, NULL, NULL, ops);
    int sizeV = nev_init + 2 * block_size;
    int len_dbl = 2 * sizeV * sizeV + 10 * sizeV + (nev_max + 2 * block_size) + nev_max * block_size;
    int len_int = 6 * sizeV + 2 * (block_size + 3);
    double *dbl_ws = calloc((size_t)len_dbl, sizeof(double));
    int *int_ws = calloc((size_t)len_int, sizeof(int));
    srand(0);

    double tol[2] = {abs_tol, rel_tol};
    EigenSolverSetup_GCG(gap_min, nev_init, nev_max, block_size, tol, max_iter, 0, 0, 0,
                         mv_ws, dbl_ws, int_ws, ops);
    GCGE_Setparameters(gap_min, auto_shift, ops);
    if (orth_method != NULL)
        EigenSolverSetParameters_GCG(0, orth_method, orth_block_size, -1, 0.0,
                                     NULL, -1, -1, 0.0,
                                     orth_method, orth_block_size, -1, 0.0,
                                     0, 0.0, 0.0, NULL, auto_shift, 0, 0.0, 0.0, ops);
    if (argc > 0)
        EigenSolverSetParametersFromCommandLine_GCG(argc, argv, ops);
    int nconv = nev;
    ops->EigenSolver(&A, matB, eval, evec, nev_given, &nconv, ops);

    memcpy(eval_out, eval, sizeof(double) * (size_t)nev_max);
    memcpy(evec_out, ev->data, sizeof(double) * (size_t)n * (size_t)nev_max);
    *nconv_out = nconv;
    *niter_out = ((GCGSolver *)ops->eigen_solver_workspace)->numIter;

    /* GCGE_Destroymvws frees dbl_ws/int_ws as well (src/ops_eig_sol_gcg.c:1919-1927). */
    GCGE_Destroymvws(mv_ws, dbl_ws, int_ws, nev_max, block_size, ops);
    ops->MultiVecDestroy(&evec, nev_max, ops);
    free(eval);
    OPS_Destroy(&ops);
    return 0;
}

int ref_gcg_solve(int n,
                  const int *a_colptr, const int *a_rowind, const double *a_val,
                  const int *b_colptr, const int *b_rowind, const double *b_val,
                  int nev, int block_size, int nev_init, int nev_max, int max_iter,
                  double abs_tol, double rel_tol, double gap_min, int auto_shift,
                  const double *x0, int nev_given,
                  double *eval_out, double *evec_out, int *nconv_out, int *niter_out)
{
    return ref_gcg_solve_opts(n, a_colptr, a_rowind, a_val, b_colptr, b_rowind, b_val, nev,
                              block_size, nev_init, nev_max, max_iter, abs_tol, rel_tol, gap_min,
                              auto_shift, x0, nev_given, eval_out, evec_out, nconv_out,
                              niter_out, NULL, 0, 0, NULL);
}

#include "ops_orth.h"
/* One call of the reference's MultiVecOrth on a column-major block x (n x m,
 * leading dimension n) through the app_ccs backend: "bgs" or "mgs" with the
 * given block size / reorthogonalisations / zero tolerance; B (CCS) may be
 * NULL.  Columns [start, *end) are orthogonalised against [0, start). */
int ref_orth(int n, int m, double *x, int start, int *end, const char *method, int block_size,
             int max_reorth, double zero_tol,
             const int *b_colptr, const int *b_rowind, const double *b_val)
{
    OPS *ops = NULL;
    OPS_Create(&ops);
    OPS_CCS_Set(ops);
    OPS_Setup(ops);
    CCSMAT B;
    void *matB = NULL;
    if (b_colptr != NULL) {
        B.data = (double *)b_val; B.i_row = (int *)b_rowind; B.j_col = (int *)b_colptr;
        B.nrows = n; B.ncols = n;
        matB = &B;
    }
    LAPACKVEC X = {x, n, m, n};
    double *ws_data = calloc((size_t)n * (size_t)m, sizeof(double));
    LAPACKVEC WS = {ws_data, n, m, n};
    double *dbl_ws = calloc((size_t)(8 * m * m + 64 * m + 1024), sizeof(double));
    if (strcmp(method, "bgs") == 0)
        MultiVecOrthSetup_BinaryGramSchmidt(block_size, max_reorth, zero_tol, (void **)&WS, dbl_ws,
                                            ops);
    else
        MultiVecOrthSetup_ModifiedGramSchmidt(block_size, max_reorth, zero_tol, (void **)&WS, dbl_ws,
                                              ops);
    ops->MultiVecOrth((void **)&X, start, end, matB, ops);
    free(ws_data);
    free(dbl_ws);
    OPS_Destroy(&ops);
    return 0;
}

#include "ops_lin_sol.h"
/* A transfer operator between adjacent levels for the app_ccs backend: P
 * (fine rows x coarse columns) and P^T, both CCS. */
typedef struct {
    CCSMAT P, PT;
} RefTransfer;

/* ops->MultiVecFromItoJ for app_ccs, which leaves the slot NULL
 * (src/ops.c:78) and ships no implementation (src/ops.c:110-112 is commented
 * out): level by level from level_i to level_j, restriction x_{l+1} = P_l^T
 * x_l and prolongation x_l = P_l x_{l+1} with app_ccs's own MatDotMultiVec
 * (rectangular CCS, app/app_ccs.c:50-139); columns [startIJ[0], endIJ[0]) of
 * multi_vec_i to [startIJ[1], endIJ[1]) of multi_vec_j, through columns
 * [0, k) of multi_vec_ws[l] at the levels in between. */
static void ref_from_i_to_j(void **P_array, int level_i, int level_j, void **mv_i, void **mv_j,
                            int *startIJ, int *endIJ, void ***mv_ws, struct OPS_ *ops)
{
    int k = endIJ[0] - startIJ[0];
    int step = level_j > level_i ? 1 : -1;
    void **src = mv_i;
    int s0 = startIJ[0], l;
    for (l = level_i; l != level_j; l += step) {
        int next = l + step;
        void **dst = next == level_j ? mv_j : mv_ws[next];
        int d0 = next == level_j ? startIJ[1] : 0;
        int start[2] = {s0, d0}, end[2] = {s0 + k, d0 + k};
        RefTransfer *t = (RefTransfer *)P_array[step > 0 ? l : next];
        ops->MatDotMultiVec(step > 0 ? (void *)&t->PT : (void *)&t->P, src, dst, start, end, ops);
        src = dst;
        s0 = d0;
    }
}

/* The reference's BlockAMG (MultiLinearSolverSetup_BlockAMG and the solver
 * it installs, src/ops_lin_sol.c:466-715) on the app_ccs backend: levels
 * 0..num_levels-1 with A_l (n[l] x n[l], CCS) and transfers P_l
 * (n[l] x n[l+1]) with their transposes, each given as three arrays per
 * level; b and x are n[0] x k column-major (x holds the initial guess and
 * receives the result); max_iter (2 num_levels entries), rate and tol (one
 * per level) and tol_type as the setup takes them.  *residual_out receives
 * the solver's residual field. */
int ref_block_amg(int num_levels, const int *n,
                  const int **a_colptr, const int **a_rowind, const double **a_val,
                  const int **p_colptr, const int **p_rowind, const double **p_val,
                  const int **pt_colptr, const int **pt_rowind, const double **pt_val,
                  int k, const double *b, double *x,
                  int *max_iter, double *rate, double *tol, const char *tol_type,
                  double *residual_out)
{
    OPS *ops = NULL;
    OPS_Create(&ops);
    OPS_CCS_Set(ops);
    OPS_Setup(ops);
    ops->MultiVecFromItoJ = ref_from_i_to_j;

    int L = num_levels, l, i;
    CCSMAT *A = calloc((size_t)L, sizeof(CCSMAT));
    RefTransfer *T = calloc((size_t)(L > 1 ? L - 1 : 1), sizeof(RefTransfer));
    void **A_array = calloc((size_t)L, sizeof(void *));
    void **P_array = calloc((size_t)(L > 1 ? L - 1 : 1), sizeof(void *));
    for (l = 0; l < L; ++l) {
        A[l].data = (double *)a_val[l]; A[l].i_row = (int *)a_rowind[l];
        A[l].j_col = (int *)a_colptr[l]; A[l].nrows = n[l]; A[l].ncols = n[l];
        A_array[l] = &A[l];
    }
    for (l = 0; l + 1 < L; ++l) {
        T[l].P.data = (double *)p_val[l]; T[l].P.i_row = (int *)p_rowind[l];
        T[l].P.j_col = (int *)p_colptr[l]; T[l].P.nrows = n[l]; T[l].P.ncols = n[l + 1];
        T[l].PT.data = (double *)pt_val[l]; T[l].PT.i_row = (int *)pt_rowind[l];
        T[l].PT.j_col = (int *)pt_colptr[l]; T[l].PT.nrows = n[l + 1]; T[l].PT.ncols = n[l];
        P_array[l] = &T[l];
    }
    void ***mv_array_ws[5];
    for (i = 0; i < 5; ++i) {
        mv_array_ws[i] = calloc((size_t)L, sizeof(void **));
        for (l = 0; l < L; ++l)
            ops->MultiVecCreateByMat(&mv_array_ws[i][l], k, &A[l], ops);
    }
    void **mv_b = NULL, **mv_x = NULL;
    ops->MultiVecCreateByMat(&mv_b, k, &A[0], ops);
    ops->MultiVecCreateByMat(&mv_x, k, &A[0], ops);
    memcpy(((LAPACKVEC *)mv_b)->data, b, sizeof(double) * (size_t)n[0] * (size_t)k);
    memcpy(((LAPACKVEC *)mv_x)->data, x, sizeof(double) * (size_t)n[0] * (size_t)k);
    double *dbl_ws = calloc((size_t)(8 * k + 64), sizeof(double));
    int *int_ws = calloc((size_t)(4 * k + 64), sizeof(int));

    MultiLinearSolverSetup_BlockAMG(max_iter, rate, tol, tol_type, A_array, P_array, L,
                                    mv_array_ws, dbl_ws, int_ws, NULL, ops);
    int start[2] = {0, 0}, end[2] = {k, k};
    ops->MultiLinearSolver(A_array[0], mv_b, mv_x, start, end, ops);
    *residual_out = ((BlockAMGSolver *)ops->multi_linear_solver_workspace)->residual;
    memcpy(x, ((LAPACKVEC *)mv_x)->data, sizeof(double) * (size_t)n[0] * (size_t)k);

    ops->MultiVecDestroy(&mv_b, k, ops);
    ops->MultiVecDestroy(&mv_x, k, ops);
    for (i = 0; i < 5; ++i) {
        for (l = 0; l < L; ++l) ops->MultiVecDestroy(&mv_array_ws[i][l], k, ops);
        free(mv_array_ws[i]);
    }
    free(dbl_ws); free(int_ws); free(A); free(T); free(A_array); free(P_array);
    OPS_Destroy(&ops);
    return 0;
}

/* One call of the reference's BlockPCG (MultiLinearSolverSetup_BlockPCG +
 * ops->MultiLinearSolver, src/ops_lin_sol.c:140-465) on the app_ccs backend:
 * A (n x n CCS) x = b for columns [sb, sb + k) of b (n x mb) into
 * [sx, sx + k) of x (n x mx, holding the initial guess), with max_iter, rate,
 * tol and tol_type ("abs", "rel", or "user" with |user_norms[i]| as the
 * norms).  *niter_out and *residual_out receive the solver record's fields. */
int ref_block_pcg(int n, const int *a_colptr, const int *a_rowind, const double *a_val,
                  int mb, double *b, int sb, int mx, double *x, int sx, int k,
                  int max_iter, double rate, double tol, const char *tol_type,
                  const double *user_norms, int *niter_out, double *residual_out)
{
    OPS *ops = NULL;
    OPS_Create(&ops);
    OPS_CCS_Set(ops);
    OPS_Setup(ops);
    CCSMAT A;
    A.data = (double *)a_val; A.i_row = (int *)a_rowind; A.j_col = (int *)a_colptr;
    A.nrows = n; A.ncols = n;
    LAPACKVEC B = {b, n, mb, n}, X = {x, n, mx, n};
    void **ws[3];
    int i;
    for (i = 0; i < 3; ++i) ops->MultiVecCreateByMat(&ws[i], k, &A, ops);
    double *dbl_ws = calloc((size_t)(6 * k + 64), sizeof(double));
    int *int_ws = calloc((size_t)(2 * k + 64), sizeof(int));
    if (user_norms != NULL)
        memcpy(dbl_ws, user_norms, sizeof(double) * (size_t)k);
    MultiLinearSolverSetup_BlockPCG(max_iter, rate, tol, tol_type, ws, dbl_ws, int_ws, NULL, NULL,
                                    ops);
    int start[2] = {sb, sx}, end[2] = {sb + k, sx + k};
    ops->MultiLinearSolver(&A, (void **)&B, (void **)&X, start, end, ops);
    BlockPCGSolver *s = (BlockPCGSolver *)ops->multi_linear_solver_workspace;
    *niter_out = s->niter;
    *residual_out = s->residual;
    for (i = 0; i < 3; ++i) ops->MultiVecDestroy(&ws[i], k, ops);
    free(dbl_ws);
    free(int_ws);
    OPS_Destroy(&ops);
    return 0;
}
