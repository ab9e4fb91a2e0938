/*
 * gcge_ops.h - the OPS plugin surface of GCGE, as exported by the GB300
 * library (libgcge_cuda.so).
 *
 * `struct OPS_` reproduces the reference's vtable member for member
 * (src/ops.h:43-152) so that code written against the reference's OPS can
 * fill it with the CUDA backend (OPS_CUDA_Set, see gcge_cuda.h) and call the
 * GPU GCG through the same entry points.  `GCGSolver` reproduces
 * src/ops_eig_sol_gcg.h:21-52 so that callers that read
 * ((GCGSolver *)ops->eigen_solver_workspace)->numIter (gcge.c:523) keep
 * working.  Both layouts are ABI contracts and must not be reordered.
 *
 * All functions keep the reference's signatures: they return void, take
 * half-open column ranges start[2]/end[2] ([0] = source x, [1] = destination
 * y), host coefficient arrays (column-major, leading dimension ldc/ldIP) and
 * opaque matrix/multivector handles.  Errors are recorded in a sticky status
 * (ops_cuda_last_error(), gcge_cuda.h) instead of assert().
 */
#ifndef GCGE_OPS_H
#define GCGE_OPS_H

#ifdef __cplusplus
extern "C" {
#endif

/* src/ops.h:43-152 */
typedef struct OPS_ {
    void   (*Printf)(const char *fmt, ...);
    double (*GetWtime)(void);
    int    (*GetOptionFromCommandLine)(const char *name, char type, void *data,
                                       int argc, char *argv[], struct OPS_ *ops);
    /* mat */
    void (*MatView)(void *mat, struct OPS_ *ops);
    void (*MatAxpby)(double alpha, void *matX, double beta, void *matY, struct OPS_ *ops);
    /* vec */
    void (*VecCreateByMat)(void **des_vec, void *src_mat, struct OPS_ *ops);
    void (*VecCreateByVec)(void **des_vec, void *src_vec, struct OPS_ *ops);
    void (*VecDestroy)(void **des_vec, struct OPS_ *ops);
    void (*VecView)(void *x, struct OPS_ *ops);
    void (*VecInnerProd)(void *x, void *y, double *inner_prod, struct OPS_ *ops);
    void (*VecLocalInnerProd)(void *x, void *y, double *inner_prod, struct OPS_ *ops);
    void (*VecSetRandomValue)(void *x, struct OPS_ *ops);
    void (*VecAxpby)(double alpha, void *x, double beta, void *y, struct OPS_ *ops);
    void (*MatDotVec)(void *mat, void *x, void *y, struct OPS_ *ops);
    void (*MatTransDotVec)(void *mat, void *x, void *y, struct OPS_ *ops);
    /* multi-vec */
    void (*MultiVecCreateByMat)(void ***multi_vec, int num_vec, void *src_mat, struct OPS_ *ops);
    void (*MultiVecCreateByVec)(void ***multi_vec, int num_vec, void *src_vec, struct OPS_ *ops);
    void (*MultiVecCreateByMultiVec)(void ***multi_vec, int num_vec, void **src_mv, struct OPS_ *ops);
    void (*MultiVecDestroy)(void ***multi_vec, int num_vec, struct OPS_ *ops);
    void (*GetVecFromMultiVec)(void **multi_vec, int col, void **vec, struct OPS_ *ops);
    void (*RestoreVecForMultiVec)(void **multi_vec, int col, void **vec, struct OPS_ *ops);
    void (*MultiVecView)(void **x, int start, int end, struct OPS_ *ops);
    void (*MultiVecLocalInnerProd)(char nsdIP, void **x, void **y, int is_vec, int *start,
                                   int *end, double *inner_prod, int ldIP, struct OPS_ *ops);
    void (*MultiVecInnerProd)(char nsdIP, void **x, void **y, int is_vec, int *start, int *end,
                              double *inner_prod, int ldIP, struct OPS_ *ops);
    void (*MultiVecSetRandomValue)(void **multi_vec, int start, int end, struct OPS_ *ops);
    void (*MultiVecAxpby)(double alpha, void **x, double beta, void **y, int *start, int *end,
                          struct OPS_ *ops);
    void (*MultiVecLinearComb)(void **x, void **y, int is_vec, int *start, int *end,
                               double *coef, int ldc, double *beta, int incb, struct OPS_ *ops);
    void (*MatDotMultiVec)(void *mat, void **x, void **y, int *start, int *end, struct OPS_ *ops);
    void (*MatTransDotMultiVec)(void *mat, void **x, void **y, int *start, int *end,
                                struct OPS_ *ops);
    void (*MultiVecQtAP)(char ntsA, char ntsdQAP, void **mvQ, void *matA, void **mvP, int is_vec,
                         int *start, int *end, double *qAp, int ldQAP, void **mv_ws,
                         struct OPS_ *ops);
    /* dense matrix ops */
    struct OPS_ *lapack_ops;
    void (*DenseMatQtAP)(char ntluA, char nsdC, int nrowsA, int ncolsA, int nrowsC, int ncolsC,
                         double alpha, double *matQ, int ldQ, double *matA, int ldA,
                         double *matP, int ldP, double beta, double *matC, int ldC,
                         double *dbl_ws);
    void (*DenseMatOrth)(double *mat, int nrows, int ldm, int start, int *end,
                         double orth_zero_tol, double *dbl_ws, int length, int *int_ws);
    /* linear solver */
    void (*LinearSolver)(void *mat, void *b, void *x, struct OPS_ *ops);
    void *linear_solver_workspace;
    void (*MultiLinearSolver)(void *mat, void **b, void **x, int *start, int *end,
                              struct OPS_ *ops);
    void *multi_linear_solver_workspace;
    /* orthonormal */
    void (*MultiVecOrth)(void **x, int start_x, int *end_x, void *B, struct OPS_ *ops);
    void *orth_workspace;
    /* multigrid */
    void (*MultiGridCreate)(void ***A_array, void ***B_array, void ***P_array, int *num_levels,
                            void *A, void *B, struct OPS_ *ops);
    void (*MultiGridDestroy)(void ***A_array, void ***B_array, void ***P_array, int *num_levels,
                             struct OPS_ *ops);
    void (*VecFromItoJ)(void **P_array, int level_i, int level_j, void *vec_i, void *vec_j,
                        void **vec_ws, struct OPS_ *ops);
    void (*MultiVecFromItoJ)(void **P_array, int level_i, int level_j, void **multi_vec_i,
                             void **multi_vec_j, int *startIJ, int *endIJ, void ***multi_vec_ws,
                             struct OPS_ *ops);
    /* eigen solver */
    void (*EigenSolver)(void *A, void *B, double *eval, void **evec, int nevGiven, int *nevConv,
                        struct OPS_ *ops);
    void *eigen_solver_workspace;
    struct OPS_ *app_ops;
} OPS;

/* src/ops_eig_sol_gcg.h:21-52 */
typedef struct GCGSolver_ {
    void *A; void *B; double sigma;
    double *eval; void **evec;
    int nevMax; double gapMin;
    int nevInit; int nevGiven; int nevConv;
    int block_size; double tol[2]; int numIterMax;
    int numIter; int sizeV;
    void **mv_ws[4]; double *dbl_ws; int *int_ws;
    int length_dbl_ws;
    int print; int printtime;
    int user_defined_multi_linear_solver;
    int check_conv_max_num;
    char initX_orth_method[8]; int initX_orth_block_size;
    int initX_orth_max_reorth; double initX_orth_zero_tol;
    char compP_orth_method[8]; int compP_orth_block_size;
    int compP_orth_max_reorth; double compP_orth_zero_tol;
    char compW_orth_method[8]; int compW_orth_block_size;
    int compW_orth_max_reorth; double compW_orth_zero_tol;
    int compW_cg_max_iter; double compW_cg_rate;
    double compW_cg_tol; char compW_cg_tol_type[8];
    int compW_cg_auto_shift; double compW_cg_shift;
    int compW_cg_order;
    int compRR_min_num; double compRR_min_gap;
    double compRR_tol;
} GCGSolver;

/* src/ops_lin_sol.h:29-40: the block-PCG parameters that
 * MultiLinearSolverSetup_BlockPCG stores; ops->multi_linear_solver_workspace
 * points at one, whose niter / residual the solve fills in. */
typedef struct BlockPCGSolver_ {
    int max_iter; double rate; double tol; char tol_type[8];
    void **mv_ws[3];  /* r p w */
    double *dbl_ws;
    int *int_ws;
    void *pc;
    void (*MatDotMultiVec)(void **x, void **y, int *start, int *end, void **z, int s,
                           struct OPS_ *ops);
    int niter; double residual;
} BlockPCGSolver;

/* src/ops_lin_sol.h:41-47: the block AMG parameters that
 * MultiLinearSolverSetup_BlockAMG stores (pointers to the caller's arrays);
 * ops->multi_linear_solver_workspace points at one between solves, and the
 * solve fills in residual (and niter, the cycles run, which the reference
 * leaves at 0). */
typedef struct BlockAMGSolver_ {
    int *max_iter; double *rate; double *tol; char tol_type[8];
    void **A_array; void **P_array; int num_levels;
    void ***mv_array_ws[5]; double *dbl_ws; int *int_ws;
    void *pc;
    int niter; double residual;
} BlockAMGSolver;

/* OPS lifetime: src/ops.c:26-149.  OPS_Setup fills Printf/GetWtime/
 * GetOptionFromCommandLine defaults; the GPU GCG needs no lapack_ops. */
void OPS_Create(OPS **ops);
void OPS_Setup(OPS *ops);
void OPS_Destroy(OPS **ops);

/* MultiVecOrth setup: src/ops_orth.h:36-41, src/ops_orth.c:395-414 (modified
 * Gram-Schmidt) and :625-641 (binary Gram-Schmidt).  Each installs the GPU
 * orthogonalisation as ops->MultiVecOrth with its parameters in
 * ops->orth_workspace: MultiVecOrth(x, start_x, &end_x, B, ops) B-orthonormalises
 * columns [start_x, end_x) of a CUDA multivector against [0, start_x) and among
 * themselves (B NULL = identity), shrinking end_x by the columns dropped as
 * dependent (B-norm below orth_zero_tol).  The binary variant follows the
 * reference's recursion and leaf choice (OrthSelf under 16 columns, else
 * OrthSelfEVP; block_size <= 0 picks the reference's default); the modified
 * variant is the GPU's blocked CGS + Cholesky-QR2 with the same dropping rule
 * (block_size unused).  mv_ws / dbl_ws are accepted for signature
 * compatibility; the device workspace belongs to ops (freed by OPS_Destroy),
 * so, unlike the reference's single static setting, each ops keeps its own. */
void MultiVecOrthSetup_ModifiedGramSchmidt(int block_size, int max_reorth, double orth_zero_tol,
                                           void **mv_ws, double *dbl_ws, struct OPS_ *ops);
void MultiVecOrthSetup_BinaryGramSchmidt(int block_size, int max_reorth, double orth_zero_tol,
                                         void **mv_ws, double *dbl_ws, struct OPS_ *ops);

/* Linear-solver setup: src/ops_lin_sol.h:41-45, src/ops_lin_sol.c:439-465.
 * Installs the GPU block conjugate gradient (src/ops_lin_sol.c:140-437) as
 * ops->MultiLinearSolver(mat, b, x, start, end, ops), solving mat x = b for
 * columns [start[0], end[0]) of b into [start[1], end[1]) of x (x holds the
 * initial guess) with the reference's per-column stopping rule: stop when the
 * residual norm is <= rate x the initial one or <= tol x norm_b (norm_b = 1
 * for "abs", ||b_i|| for "rel", |dbl_ws[i]| for "user"), or after max_iter
 * steps.  With MatDotMultiVec NULL and an "abs"/"rel" tolerance the solve is
 * one persistent kernel launch per 40 columns on the CUDA matrix `mat`; with
 * an operator callback (e.g. the shifted product of GCG's ComputeW) or
 * "user" norms, the reference's loop runs step for step on the device
 * multivectors, calling the callback on the same column ranges with the same
 * workspace arguments; mv_ws[0..2] (r, p, w: CUDA multivectors at least as
 * wide as the block) are then required.  pc and int_ws are stored and unused,
 * as in the reference.  Each ops keeps its own setting (the reference keeps
 * one static setting per process).  Failures go to ops_cuda_last_error(). */
void MultiLinearSolverSetup_BlockPCG(int max_iter, double rate, double tol, const char *tol_type,
                                     void **mv_ws[3], double *dbl_ws, int *int_ws, void *pc,
                                     void (*MatDotMultiVec)(void **x, void **y, int *start,
                                                            int *end, void **z, int s,
                                                            struct OPS_ *ops),
                                     struct OPS_ *ops);

/* Block AMG setup: src/ops_lin_sol.h:48-53, src/ops_lin_sol.c:686-715.
 * Installs the V-cycle of src/ops_lin_sol.c:466-685 as
 * ops->MultiLinearSolver(mat, b, x, start, end, ops) over the caller's
 * hierarchy: A_array[l] CUDA matrices (l < num_levels, A_array[0] the
 * operator), P_array[l] transfers of n_l x n_{l+1} from
 * CUDA_TransferCreateFromCCS, and mv_array_ws[i][l] CUDA multivectors of
 * level l at least as wide as the block (0, 1: the coarse right-hand side and
 * solution, levels >= 1; 2, 3, 4: the level's residual and smoothing
 * workspaces).  Each level smooths with MultiLinearSolverSetup_BlockPCG
 * (max_iter[2l+1] before and max_iter[2l+2] after the coarse correction,
 * rate[l], tol[l], tol_type); cycles repeat until the residual field of the
 * last level-0 smoothing is below tol[0] or after max_iter[0] cycles.  The
 * arrays are read at every solve (the caller keeps them alive).  ops must
 * provide MultiVecFromItoJ (OPS_CUDA_Set installs CUDA_MultiVecFromItoJ).
 * Failures go to ops_cuda_last_error(). */
void MultiLinearSolverSetup_BlockAMG(int *max_iter, double *rate, double *tol,
                                     const char *tol_type, void **A_array, void **P_array,
                                     int num_levels, void ***mv_array_ws[5], double *dbl_ws,
                                     int *int_ws, void *pc, struct OPS_ *ops);

/* GCG entry points: src/ops_eig_sol_gcg.c:1565-1628 (Setup), :1684-1741
 * (SetParameters), :1865-1877 (GCGE_Create), :1878-1918 (GCGE_Setparameters),
 * :1919-1927 (GCGE_Destroymvws), :1630-1680 (workspace create/destroy).
 * EigenSolverSetup_GCG installs the GPU GCG as ops->EigenSolver; the
 * multivector workspaces must come from a CUDA-backed ops (OPS_CUDA_Set).
 * dbl_ws / int_ws are accepted for signature compatibility; the GPU solver
 * keeps its small dense state in its own per-ops context. */
void EigenSolverSetup_GCG(double gapMin, int nevInit, int nevMax, int block_size, double tol[2],
                          int numIterMax, int print, int printtime,
                          int user_defined_multi_linear_solver, void **mv_ws[4], double *dbl_ws,
                          int *int_ws, struct OPS_ *ops);
void EigenSolverCreateWorkspace_GCG(int nevInit, int nevMax, int block_size, void *mat,
                                    void ***mv_ws, double **dbl_ws, int **int_ws,
                                    struct OPS_ *ops);
void EigenSolverDestroyWorkspace_GCG(int nevInit, int nevMax, int block_size, void *mat,
                                     void ***mv_ws, double **dbl_ws, int **int_ws,
                                     struct OPS_ *ops);
void EigenSolverSetParameters_GCG(
    int check_conv_max_num, const char *initX_orth_method, int initX_orth_block_size,
    int initX_orth_max_reorth, double initX_orth_zero_tol, const char *compP_orth_method,
    int compP_orth_block_size, int compP_orth_max_reorth, double compP_orth_zero_tol,
    const char *compW_orth_method, int compW_orth_block_size, int compW_orth_max_reorth,
    double compW_orth_zero_tol, int compW_cg_max_iter, double compW_cg_rate, double compW_cg_tol,
    const char *compW_cg_tol_type, int compW_cg_auto_shift, int compRR_min_num,
    double compRR_min_gap, double compRR_tol, struct OPS_ *ops);
/* src/ops_eig_sol_gcg.c:1743-1862 (declared at src/ops_eig_sol_gcg.h:83): the
 * "-gcge_*" options of argv override the solver parameters, e.g.
 * -gcge_compW_orth_method bgs, -gcge_compW_cg_order 2 (ComputeW12).
 * -gcge_compRR_min_gap is read as a double; the usage table is not printed. */
void EigenSolverSetParametersFromCommandLine_GCG(int argc, char *argv[], struct OPS_ *ops);
void GCGE_Create(void *A, int nevMax, int block_size, int nevInit, void ***gcg_mv_ws,
                 double *dbl_ws, int *int_ws, struct OPS_ *ops);
void GCGE_Setparameters(double gapMin, int shift, struct OPS_ *ops);
void GCGE_Destroymvws(void ***gcg_mv_ws, double *dbl_ws, int *int_ws, int nevMax, int block_size,
                      struct OPS_ *ops);

#ifdef __cplusplus
}
#endif
#endif /* GCGE_OPS_H */
