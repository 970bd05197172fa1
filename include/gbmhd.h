/*
 * gbmhd.h — C ABI of the GB300 inductionless-MHD Newton assembly and solve.
 *
 * Drop-in for the hot path of GridapMHD.jl: the Newton Jacobian/residual
 * assembly of the H1-HDiv weak form (u Q2, p dP1, j RT1, φ dQ1) and the sparse
 * linear solve inside each Newton step.  A Julia host keeps
 * `GridapMHD.main(params)` / `hunt(...)` and reaches this library with `ccall`
 * through a new `:gb300` solver symbol.
 *
 * Interfaces replaced (paths inside GridapMHD.jl):
 *   gbmhd_create        SparseMatrixAssembler + FEOperator set-up, src/main.jl:218-224,
 *                       with the spaces of src/fespaces.jl:13-114 passed as cell dof ids
 *   gbmhd_assemble      residual(op,xh) / jacobian(op,xh) timing entry, src/main.jl:156-165,
 *                       integrands of src/weakforms.jl:255-312 and :721-733
 *   gbmhd_newton_solve  _solver(::Val{:julia}) NewtonSolver + the linear solve,
 *                       src/main.jl:181-186 and :275; Badia2024Solver FGMRES +
 *                       block-triangular preconditioner, src/Solvers/badia2024.jl:2-48
 *   gbmhd_adjoint       no counterpart in the reference (discrete adjoint of the solve)
 *   gbmhd_param_gradient_noalloc  no counterpart in the reference (the adjoint's
 *                       parameter gradient from a given λ, without device allocation)
 *   gbmhd_get_csr       the assembled SparseMatrixCSR (pattern + values), for parity checks
 *   gbmhd_hunt_errors   the post-processing of hunt(): error and solution norms against the
 *                       analytic Hunt solution, src/Applications/hunt.jl:238-260 with
 *                       analytical_hunt_u/j of :372-457
 *
 * Conventions
 *   - All host pointers are owned by the caller and only read during the call.
 *   - Status: 0 ok; >0 not converged (report filled); <0 invalid input or CUDA error.
 *     gbmhd_last_error() returns the message of the last failing call on a context.
 *   - One context per host thread; calls on a context are serialised on its
 *     own CUDA stream.
 *   - Local dof layout of a cell (129 slots):
 *       [0,81)   u, component-major c*27 + n, n = a + 3b + 9c over Lagrange nodes ξ ∈ {0,½,1}³
 *       [81,85)  p, P1 nodal at (0,0,0),(1,0,0),(0,1,0),(0,0,1)
 *       [85,121) j, RT1: d*12 + q + 3*(l1 + 2*l2), ψ = L2_q(ξ_d) L1_l1 L1_l2 e_d
 *       [121,129) φ, Q1 nodal at the 8 vertices (a + 2b + 4c)
 *     Local vertices are ordered a + 2b + 4c (x fastest), local faces axis*2 + side.
 */
#ifndef GBMHD_H
#define GBMHD_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBMHD_NDOF_CELL 129

typedef struct gbmhd_ctx gbmhd_ctx;

/* Cells of the mesh: trilinear hexahedra given by their 8 vertex coordinates
 * (Gridap: get_cell_coordinates(get_grid(model))). */
typedef struct {
  int64_t ncells;
  const double* cell_coords;   /* [ncells][8][3] */
} gbmhd_mesh;

/* Per-field dof numbering (Gridap: get_cell_dof_ids of each single-field space).
 * Free ids are field-local and >= 0; Dirichlet slots hold -(id+1). */
typedef struct {
  int64_t nfree[4];            /* u, p, j, φ free dofs; global vector is [u;p;j;φ] */
  int64_t ndir[4];             /* Dirichlet dofs per field */
  const int32_t* cell_dofs;    /* [ncells][129] */
  const double* dir_values[4]; /* Dirichlet values per field (NULL = zero) */
  const int8_t* cell_sign_j;   /* [ncells][36] orientation ±1 of the RT dofs (NULL = +1) */
} gbmhd_dofmap;

/* Physical parameters (src/weakforms.jl:71-83, :137-178). */
typedef struct {
  double alpha, beta, gamma, sigma;
  double B[3];
  double f[3];                 /* body force when f_cell is NULL */
  double g[3];                 /* Ohm's-law right-hand side */
  double zeta_u, zeta_j;       /* augmented-Lagrangian weights */
  int32_t convection;          /* 0 :none, 1 :picard, 2 :newton */
  const double* f_cell;        /* [ncells][3] cellwise body force, or NULL */
  /* boundary facets carrying the thin-wall law and/or a weak potential */
  int64_t nfacets;
  const int32_t* facet_cell;
  const int8_t* facet_lface;   /* local face axis*2 + side */
  const double* facet_tau;     /* penalty τ (NULL = 0) */
  const double* facet_cw;      /* wall conductance ratio (NULL = 0) */
  const double* facet_jw;      /* prescribed wall current (NULL = 0) */
  const double* facet_phi0;    /* weak potential value (NULL = 0) */
} gbmhd_params;

/* Precision of the element matrices and of the preconditioner.
 *   GBMHD_FP64:        FP64 Jacobian and FP64 factors
 *   GBMHD_MIXED:       FP32 element matrices and FP32 factors (the preconditioner); the
 *                      FGMRES operator is the FP64 Jacobian, the residual FP64
 *   GBMHD_MIXED_F64OP: FP32 factors of the FP64 Jacobian; FP64 operator
 * In every mode the residual, the Krylov vectors and the Newton update are FP64. */
enum { GBMHD_FP64 = 0, GBMHD_MIXED = 1, GBMHD_MIXED_F64OP = 2 };

/* Preconditioner of the FGMRES linear solve.
 *   GBMHD_PC_MONOLITHIC: nested-dissection multifrontal factorization of the whole
 *     Jacobian (the direct solve of the :julia solver, used as a preconditioner).  Each
 *     subdomain hands one p and one φ dof (its constant modes) to its parent; the two
 *     global ones are regularised in the root by −diag(mass) at the Schur scale.
 *   GBMHD_PC_BADIA2024: upper block-triangular [(u,j) | p | φ] with scaled mass blocks
 *     and a multifrontal (u,j) factorization (src/Solvers/badia2024.jl:2-48); needs the
 *     augmented-Lagrangian weights ζᵤ, ζⱼ > 0 to converge. */
enum { GBMHD_PC_MONOLITHIC = 0, GBMHD_PC_BADIA2024 = 1 };

typedef struct {
  int32_t precision;           /* GBMHD_FP64, GBMHD_MIXED or GBMHD_MIXED_F64OP */
  int32_t max_newton;          /* Newton iteration cap (reference :niter) */
  double newton_rtol;          /* ‖r‖ ≤ max(atol, rtol‖r0‖) */
  double newton_atol;
  int32_t restart;             /* FGMRES restart length m (reference :niter_ls) */
  int32_t max_linear;          /* FGMRES iteration cap per Newton step */
  double linear_rtol;          /* relative tolerance of each linear solve */
  int32_t verbose;
  int32_t preconditioner;      /* GBMHD_PC_MONOLITHIC or GBMHD_PC_BADIA2024 */
} gbmhd_solve_opts;

typedef struct {
  int32_t newton_iters;
  int32_t linear_iters;        /* summed over Newton steps */
  int32_t converged;
  double initial_residual, final_residual;
  double time_assembly_s, time_setup_pc_s, time_linear_s, time_total_s;
  double residual_history[64]; /* ‖r‖ after each Newton step (first = initial) */
  int32_t pc_refactorizations; /* mixed modes: FP32 factorizations redone after a linear solve
                                  stagnated (0 in a normal solve) */
} gbmhd_report;

/* Objective J(x) of the adjoint: a linear functional of the free vector,
 * J = ∫_plane u_z dA (flow rate) or a pressure drop, given by its gradient. */
typedef struct {
  const double* dJdx;          /* [ndofs] ∂J/∂x, host array */
  int32_t n_theta_cells;       /* >0: also return dJ/d f_z for every cell */
} gbmhd_objective;

/* Analytic Hunt solution for gbmhd_hunt_errors (src/Applications/hunt.jl:238-245). */
typedef struct {
  double L;                    /* half-width of the duct: a = b = L */
  double mu;                   /* ρν */
  double grad_pz;              /* −f_z/ρ */
  double sigma;
  double Ha;
  int32_t nsums;               /* Fourier terms k = 0..nsums; the *_ref norms use k = 0..2·nsums */
  double u_scale;              /* physical u = u_scale · the solved u (reference: u0) */
  double j_scale;              /* physical j = j_scale · the solved j (reference: σ u0 B0) */
  double length_scale;         /* physical x = length_scale · mesh x (reference: L, _warp at :352) */
} gbmhd_hunt_analytic;

int gbmhd_version(void);

int gbmhd_create(gbmhd_ctx** out, const gbmhd_mesh* mesh, const gbmhd_dofmap* dofs,
                 const gbmhd_params* params);

/* Replace the physical parameters (same mesh and dofs). */
int gbmhd_set_params(gbmhd_ctx* ctx, const gbmhd_params* params);

/* Sizes: total free dofs and Jacobian nonzeros. */
int gbmhd_sizes(const gbmhd_ctx* ctx, int64_t* ndofs, int64_t* nnz, int64_t* ncells);

/* Residual r(x) (FP64) and, if want_jacobian, the Jacobian at x in the given
 * precision, kept on the device.  x_free and r_out are host arrays [ndofs];
 * r_out may be NULL. */
int gbmhd_assemble(gbmhd_ctx* ctx, const double* x_free, double* r_out, int32_t want_jacobian,
                   int32_t precision);

/* Same with device pointers (inputs resident in HBM, no host traffic). */
int gbmhd_assemble_device(gbmhd_ctx* ctx, const double* d_x_free, double* d_r_out,
                          int32_t want_jacobian, int32_t precision);

/* Copy the last assembled Jacobian to the host: rowptr [ndofs+1], col [nnz], val [nnz]
 * (FP64; an FP32 Jacobian is widened).  Any pointer may be NULL. */
int gbmhd_get_csr(gbmhd_ctx* ctx, int64_t* rowptr, int32_t* col, double* val);

/* Newton solve from x_inout (host, [ndofs]) to convergence. */
int gbmhd_newton_solve(gbmhd_ctx* ctx, double* x_inout, const gbmhd_solve_opts* opts,
                       gbmhd_report* report);

/* Same on a device-resident vector. */
int gbmhd_newton_solve_device(gbmhd_ctx* ctx, double* d_x_inout, const gbmhd_solve_opts* opts,
                              gbmhd_report* report);

/* Discrete adjoint at a converged state x (host [ndofs]): solves Jᵀλ = ∂J/∂x and
 * returns dJ/dθ = −λᵀ ∂R/∂θ in dJ_dtheta: [0] d/dγ, [1] d/d(cw) (all thin-wall
 * facets together), [2] d/dα, [3] d/dβ, [4 .. 4+ncells) d/d f_z per cell (when
 * n_theta_cells > 0; ntheta must then be ≥ 4 + ncells, else ≥ 4).  Ha enters through
 * γ = Ha²/Re in the CFD scaling (src/Applications/hunt.jl:125-128) and through α = Re/Ha²,
 * β = 1/Ha² in the MHD scaling (src/Applications/expansion.jl:113-123); the host applies
 * the chain rule.  lambda_out (host [ndofs]) may be NULL. */
int gbmhd_adjoint(gbmhd_ctx* ctx, const double* x_free, const gbmhd_objective* obj,
                  const gbmhd_solve_opts* opts, double* dJ_dtheta, int64_t ntheta, double* lambda_out,
                  gbmhd_report* report);

/* No counterpart in the reference.  dJ/dθ = −λᵀ ∂R/∂θ for θ = (γ, cw) from a device
 * state d_x [ndofs] and a device adjoint vector d_lambda [ndofs] (from gbmhd_adjoint's
 * lambda_out, or the host's own solve of Jᵀλ = ∂J/∂x), written to d_out [2] on the
 * context's stream; the call returns without waiting for it.
 * For hosts that may not allocate device memory inside their loop (an optimiser or
 * sampler whose device memory is held by its own pool, an embedded solver that is not
 * allowed to call cudaMalloc/cudaFree after set-up): this call allocates nothing.  Its
 * scratch is a file-scope device array with room for 262,144 cells and 65,536
 * thin-wall facets (2.5 MiB per device); larger contexts are rejected with -1 and a
 * message.  Every scratch slot that a call reads it has written first, so nothing
 * needs zeroing.  The scratch is shared by every context on a device: calls that
 * overlap on the GPU (several streams or host threads) race.  The first call on a
 * device looks up the array's address with that device current; make it before any
 * stream capture.  The context's device must be the current device (else -1).  The
 * address stays cached until the process exits, so a cudaDeviceReset invalidates it.
 * In the MHD scaling (α = 1/N, β = 1/Ha²) Ha does not enter through γ: there dJ/dγ is
 * not dJ/dHa, and gbmhd_adjoint's dJ/dα and dJ/dβ are needed for it. */
int gbmhd_param_gradient_noalloc(gbmhd_ctx* ctx, const double* d_x, const double* d_lambda, double* d_out);

/* The CUDA stream (cudaStream_t) every call on this context is issued on; a
 * host can record its own events on it to time the library's kernels. */
void* gbmhd_get_stream(const gbmhd_ctx* ctx);

/* Diagnostic: relative error of the (u,j)-block direct solve of the preconditioner,
 * ‖x − A_uj⁻¹(A_uj x)‖/‖x‖ for a seeded random x, with the Jacobian assembled at the
 * device state d_state in the given precision. */
int gbmhd_diag_uj_solve_error(gbmhd_ctx* ctx, const double* d_state, int32_t precision, double* err);

/* Post-processing of hunt() (src/Applications/hunt.jl:238-260) on the device: with the
 * free vector x_free (host) and the mesh's Dirichlet values, out[9] receives
 *   {eu_h1, eu_l2, ej_l2, eu_ref_h1, eu_ref_l2, ej_ref_l2, uh_h1, uh_l2, jh_l2}
 * where eu = u_analytic − u_h and ej = j_analytic − j_h with nsums (…_ref: 2·nsums) Fourier
 * terms, integrated with 4 Gauss points per direction (degree 2(order+1) = 6). u_h and j_h
 * are the solved fields times u_scale and j_scale; their values at the reference points
 * of a cell do not change with length_scale, their gradients scale by 1/length_scale. */
int gbmhd_hunt_errors(gbmhd_ctx* ctx, const double* x_free, const gbmhd_hunt_analytic* a, double* out);

/* The solution at the 27 Q2 nodes ξ ∈ {0, ½, 1}³ of every cell (node n = a + 3b + 9c), on the
 * device, for field output of order 2 as hunt(..., vtk=true) writes it
 * (src/Applications/hunt.jl:263-273): out [ncells][27][13] receives per node the physical
 * point (3), u_h (3), p_h, j_h (3, contravariant Piola map), φ_h, div u_h and div j_h.
 * x_free is the host free vector [ndofs]; the Dirichlet values are the context's. */
int gbmhd_node_fields(gbmhd_ctx* ctx, const double* x_free, double* out);

/* Diagnostics: multifrontal solves (preconditioner applications) timed with CUDA events
 * on the context stream since the last call, their total device time in seconds, and
 * the factor bytes one solve reads (padding excluded); resets the counters. */
int gbmhd_sweep_stats(gbmhd_ctx* ctx, int64_t* applies, double* seconds, double* bytes_per_apply);

/* Diagnostic environment variables.  None is needed in normal use; without them the
 * library's behaviour is fixed.  They exist for measurements and for tests that drive
 * rarely taken paths on purpose.
 *   GBMHD_PC_EPS32, GBMHD_PC_EPS64  scale of the root's −ε·diag(mass) regularisation of the
 *                                   global p and φ pivots (FP32 factors: default 1e-3; FP64: 1)
 *   GBMHD_ELIM_ORDER                field order of elimination inside a front, both precisions
 *                                   (default "ujfp" for FP32 factors, "jufp" for FP64)
 *   GBMHD_STAG_ITERS, GBMHD_STAG_REL  the mixed-precision stagnation test: a linear solve
 *                                   that has run GBMHD_STAG_ITERS iterations (default 100) with
 *                                   its relative residual still above GBMHD_STAG_REL (default
 *                                   0.5) triggers the refactorization / FP64 fallback
 *   GBMHD_PIVOT_KERNEL              force one pivot-block inverse kernel of the FP32 factors
 *                                   (the variants of gbmhd_diag_pivot_inverse; read per factorization)
 *   GBMHD_MF_LEVEL_TIMES            print each factorization's per-level device time (CUDA
 *                                   events) and host issue time to stderr (levels in sequence)
 *   GBMHD_GAUGE_PROJECTION          0: keep the constant-pressure component of the FGMRES
 *                                   directions (removed by default when the all-ones p vector is
 *                                   a null vector of the Jacobian)
 *   GBMHD_SWEEP_GRAPHS              0: launch the kernels of each preconditioner application one
 *                                   by one instead of replaying them as a CUDA graph (for per-kernel
 *                                   profiling; read when a context first factors; default 1)
 *   GBMHD_SWEEP_BRANCHES            0: substitute and factor the level groups of one tree height
 *                                   one after another instead of side by side on branch streams
 *                                   (read when a context first factors; default 1)
 *   GBMHD_SWEEP_WAIT_LIMIT          spin limit of the TMA solve sweeps' mbarrier waits, read
 *                                   when a context first factors (default 4,194,304); a wait
 *                                   that runs out drains its copies and makes the Newton step
 *                                   or the adjoint return -3 */

/* Diagnostic: relative difference ‖y32 − y64‖/‖y64‖ of y = P⁻¹b (transpose = 0) or P⁻ᵀb
 * (transpose = 1) for a seeded random b, with the monolithic preconditioner factored in FP32
 * (from the FP32 Jacobian) and in FP64, both assembled at the device state d_state. */
int gbmhd_diag_pc_compare(gbmhd_ctx* ctx, const double* d_state, int32_t transpose, double* err);

/* Diagnostic: the float-float Gauss-Jordan inverse of the FP32 factorization's NB x NB
 * (64 x 64) diagonal pivot blocks, with partial pivoting inside the block: for each of `count`
 * column-major n x n fronts in the device buffer F, the leading kb x kb block's inverse goes
 * to P (count blocks of 64 x 64, column-major, zero outside kb x kb).  variant selects the
 * kernel (0: 16 column groups of 64 rows, 1: 4 column groups, 2: block in shared memory,
 * 3: one column pair per warp, one barrier per column step); all give the same bits.  After
 * one checked launch, `reps` more are timed with CUDA events (*ms_per_launch).  Synchronises
 * the device; *status = 1 if a block was singular.  No counterpart in the reference (its
 * dense kernels are UMFPACK's, src/main.jl:181-186). */
int gbmhd_diag_pivot_inverse(int32_t variant, int32_t count, int32_t n, int32_t kb, const float* F, float* P,
                             int32_t reps, double* ms_per_launch, int32_t* status);

/* Diagnostic: the FP32 strided-batched GEMM of the factorization's dense updates, on the
 * tcgen05 tensor cores (three-way BF16 splits of each operand, six cross products, FP32
 * accumulation in tensor memory): C = alpha·A·B + beta·C for `batch` column-major problems on
 * device buffers (A m x k, B k x n, C m x n, strides sA, sB, sC between problems), 1 ≤ k ≤ 128.
 * Synchronises the device; *status = 0, or 2 if a tensor-core wait timed out.  No counterpart
 * in the reference (its dense kernels are UMFPACK's, src/main.jl:181-186). */
int gbmhd_diag_tc_gemm(int32_t m, int32_t n, int32_t k, float alpha, const float* A, int32_t lda, int64_t sA,
                       const float* B, int32_t ldb, int64_t sB, float beta, float* C, int32_t ldc, int64_t sC,
                       int32_t batch, int32_t* status);

/* Diagnostics: kernels launched by this library and cuBLAS GEMM calls it made
 * since it was loaded (all contexts together). */
int gbmhd_counters(int64_t* kernel_launches, int64_t* gemm_calls);

const char* gbmhd_last_error(const gbmhd_ctx* ctx);
void gbmhd_destroy(gbmhd_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif /* GBMHD_H */
