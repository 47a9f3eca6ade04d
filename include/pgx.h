/*
 * pgx.h -- C ABI of libpypde_gb300.so, the GB300 (sm_103a) FP64 kernels behind
 * the pypde spectral-Galerkin time step.
 *
 * Conventions (all entry points):
 *   - Every pointer to double is DEVICE memory owned by the caller, float64.
 *     Host pointers are only taken where a parameter says "host".
 *   - 2-D arrays are strided views: element (i, j) lives at ptr[i*s0 + j*s1]
 *     (strides in elements).  "axis" 0 means the 1-D operation runs along i
 *     (the reference's axis 0 / x), 1 along j (axis 1 / y).
 *   - Launches are asynchronous on the given cudaStream_t (passed as void*,
 *     NULL = legacy default stream).  Nothing synchronises.
 *   - Return value: 0 on success, otherwise a PGX_E* code; pgx_error_string()
 *     describes it.  No C++ exception crosses the ABI.
 *   - Thread-compatible: plan creation is internally locked; a plan may be used
 *     from several host threads on different streams.
 *
 * The entry points replace the reference's f2py / SciPy call sites; each
 * declaration names the reference interface it stands in for (file:line of
 * pypde by preiter93).
 */
#ifndef PGX_H
#define PGX_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ errors */
#define PGX_OK 0
#define PGX_E_ARG 1          /* bad shape, stride, length or enum */
#define PGX_E_CUDA 2         /* a CUDA runtime call failed (see pgx_last_cuda_error) */
#define PGX_E_SMEM 3         /* the requested tile does not fit in shared memory */
#define PGX_E_PLAN 4         /* null or destroyed plan handle */
#define PGX_E_SINGULAR 5     /* zero pivot while factoring a banded matrix */

const char* pgx_error_string(int code);
int pgx_last_cuda_error(void);
int pgx_version(void);

/* --------------------------------------------------------- line programs
 * A line program runs a sequence of 1-D operations on tiles of lines held in
 * shared memory: every CTA loads `tb` lines of one instance, applies the ops,
 * and stores results.  One launch = one pass along one axis.  The fused RBC
 * step and every single-operation entry point below are line programs.
 */
#define PGX_MAX_ARR 24
#define PGX_MAX_MAT 16
#define PGX_MAX_LEN 16
#define PGX_MAX_PAR 16
#define PGX_MAX_OPS 96
#define PGX_MAX_SLOTS 8
#define PGX_LMAX 2112        /* longest line (elements) a program may hold */

typedef struct pgx_array {
  double* ptr;
  int64_t s0, s1;            /* strides of dims 0 and 1, in elements */
  int32_t n0, n1;            /* extents */
} pgx_array;

typedef struct pgx_instance {
  pgx_array arr[PGX_MAX_ARR];      /* arrays the ops load from / store to */
  const double* mat[PGX_MAX_MAT];  /* operator tables (device) */
  int32_t len[PGX_MAX_LEN];        /* symbolic lengths */
  double par[PGX_MAX_PAR];         /* per-instance scalars */
} pgx_instance;

enum pgx_opcode {
  PGX_OP_LOAD = 1,      /* slot a = alpha * arr, logical length len          */
  PGX_OP_LOAD_ADD = 2,  /* slot a += alpha * arr                             */
  PGX_OP_LOAD_MUL = 3,  /* slot a *= alpha * arr                             */
  PGX_OP_STORE = 4,     /* arr = alpha * slot a                              */
  PGX_OP_STORE_ADD = 5, /* arr += alpha * slot a                             */
  PGX_OP_SCALE = 6,     /* slot a *= alpha                                   */
  PGX_OP_AXPY = 7,      /* slot a += alpha * slot b                          */
  PGX_OP_MUL = 8,       /* slot a *= alpha * slot b                          */
  PGX_OP_COPY = 9,      /* slot a = alpha * slot b                           */
  PGX_OP_SETLEN = 10,   /* zero-pad / truncate slot a to len                 */
  PGX_OP_STENCIL = 11,  /* slot a (M) = S slot a (M+2); mat: S[i+2,i]        */
  PGX_OP_STENCIL_T = 12,/* slot a (N) = S^T slot a (N-2); mat: S[i+2,i]      */
  PGX_OP_TDMA2 = 13,    /* slots a..a+b-1 = (S^T S)^-1 slot; mat: (a,rden,w) per i */
  PGX_OP_DIFF = 14,     /* slots a..a+b-1 = D^k slot (Chebyshev recurrence)  */
  PGX_OP_DCT = 15,      /* slots a..a+b-1 (one length) = DCT-I of themselves, all slots through each
                           phase together; k = mode; mat: twiddles */
  PGX_OP_BANDED = 17,   /* slot a = A slot a; k diagonals from offset b step 2, rows len; mat [k][rows] */
  PGX_OP_DENSE = 18,    /* slot a = A slot a; A is len x slen row-major       */
  PGX_OP_FDMA = 19,     /* in-place -2/0/+2/+4 LU solve of slots a..a+b-1, table mat+s: [l|dinv|u1|u2] */
  PGX_OP_POISSON = 20,  /* like FDMA with per-line factors (line j at j*4*n)  */
  PGX_OP_ZERO00 = 21,   /* element 0 of the instance's line 0 = 0            */
  PGX_OP_DIFF_T = 22,   /* slots a..a+b-1 = (D^T)^k slot (adjoint of DIFF)   */
  PGX_OP_FDMA_T = 23,   /* A^T x = b with the FDMA factors (adjoint of FDMA) */
  PGX_OP_POISSON_T = 24 /* per-line transposed sweep (adjoint of POISSON)    */
};

/* DCT modes; FWD_T and BWD_T are the exact transposes (adjoints) of FWD and BWD. */
enum pgx_dct_mode { PGX_DCT_RAW = 0, PGX_DCT_FWD = 1, PGX_DCT_BWD = 2, PGX_DCT_FWD_T = 3, PGX_DCT_BWD_T = 4 };
/* op.k of DCT: the mode in the low bits; PGX_DCT_CTA runs an even-length transform with its
 * phases spread over the whole CTA (block barriers between FFT stages) instead of one warp per
 * line pair.  PGX_DCT_SLOT runs the FFT of a one-slot op (b <= 1) in the slot's own lines and the
 * spare slot instead of separate buffers; it needs an even tile (tb) and a length n whose n - 1 is
 * even with an FFT stage count that can be made odd (n - 1 = 2^p 3^b with p >= 2, or p = 1 and b
 * even), and refuses other lengths (NaN).  When every DCT op of a program has it, the program
 * takes no FFT buffers of shared memory. */
#define PGX_DCT_MODE_MASK 7
#define PGX_DCT_CTA 8
#define PGX_DCT_SLOT 16

/* Chain ops (DIFF, TDMA2, FDMA) act on the b consecutive slots a..a+b-1 at
 * once (b <= 1: slot a only); BANDED uses b as its first diagonal offset.
 * op.k of TDMA2 / FDMA / FDMA_T / POISSON / POISSON_T: PGX_CHAIN_WARP selects one
 * warp per (line, parity) chain with a warp-parallel scan instead of one thread
 * per chain (for passes with few lines). */
#define PGX_CHAIN_WARP 1
/* op.k of DENSE: PGX_DENSE_MMA runs the contraction on the FP64 tensor cores (DMMA,
 * 8 x 8 x 4 tiles: rows x lines x columns) instead of one FMA chain per output. */
#define PGX_DENSE_MMA 2
/* Largest CTA: 1024 threads, 768 for programs with DCT ops (their kernel is compiled for up
 * to 80 registers a thread; the kernel without the FFT code for 64). */
#define PGX_MAX_THREADS 1024
#define PGX_MAX_THREADS_FFT 768
typedef struct pgx_op {
  int16_t code, a, b, arr, mat, len, par, k;
  double alpha;                    /* scalar; multiplied by par[par] when par >= 0 */
} pgx_op;

typedef struct pgx_program {
  int32_t axis;                    /* 0 or 1 */
  int32_t lines_len;               /* len[] index: number of lines of this pass */
  int32_t tb;                      /* lines per CTA */
  int32_t lcap;                    /* per-line capacity in shared memory (odd) */
  int32_t nslots;                  /* slots used (<= PGX_MAX_SLOTS) */
  int32_t nops;
  int32_t fft_n;                   /* longest DCT length in the program, 0 if none */
  int32_t nthreads;                /* CTA size (multiple of 32, <= PGX_MAX_THREADS; with DCT ops
                                      <= PGX_MAX_THREADS_FFT) */
  pgx_op ops[PGX_MAX_OPS];
} pgx_program;

/* Shared-memory bytes a program needs per CTA. */
int64_t pgx_program_smem(const pgx_program* prog);

/* Run one pass of a single instance.  Both structs are HOST memory, passed to
 * the kernel by value. */
int pgx_run(const pgx_program* prog, const pgx_instance* inst, void* stream);

/* The checks pgx_run applies to a program and an instance descriptor (both
 * HOST memory), without a launch and without a device: array extents and
 * lengths within the slot capacity, the tables the ops read present.  Returns
 * PGX_OK or PGX_E_ARG.  The shared-memory capacity is checked at launch. */
int pgx_check_instance(const pgx_program* prog, const pgx_instance* inst);

/* Run one pass over many instances.  `d_insts` (ninst entries) and `d_work`
 * (nwork (instance, tile) int32 pairs) are DEVICE memory, which this call does
 * not read: every descriptor must pass pgx_check_instance (on its host copy,
 * before the upload) and every work pair must name an entry of `d_insts` and a
 * tile below ceil(lines / prog->tb) of it. */
int pgx_run_batched(const pgx_program* prog, const pgx_instance* d_insts,
                    const int32_t* d_work, int32_t nwork, void* stream);

/* ------------------------------------------------------- persistent steps
 * No counterpart in the reference (its time loop is integrator.py:14-32, one
 * instance, one operation at a time).  Many passes of many instances -- whole
 * time steps of a batch -- in ONE launch: every CTA takes the next work item
 * from a queue (an atomic counter over `items`, which are in an order where
 * every item comes after the items it depends on), waits until the counter it
 * depends on has reached its target, runs the item's program on one tile of
 * one instance descriptor, and adds one to the counter it completes.  An
 * instance starts its next pass (or its next step) as soon as its own previous
 * pass is complete, not when every instance's is.
 *
 * Item fields: prog (index into the programs), desc (index into the
 * descriptors), tile, wait (counter index, or -1: no dependency), need (the
 * count `wait` must reach), done (counter index completed by this item).
 * A wait that has not been satisfied after `spin_limit` SM clock cycles ends
 * the launch with PGX_PERSIST_TIMEOUT in state[1] and the item index in
 * state[2]; an item with an out-of-range index ends it with
 * PGX_PERSIST_BAD_ITEM.  The call resets the `ncounters` counters and the
 * three state words (next item, error, where) on `stream` before the launch,
 * so it can be recorded in a CUDA graph and replayed; pgx_persist_error reads
 * the error word (synchronising the stream).
 *
 * h_progs (HOST) are checked like pgx_run's programs; d_progs must hold the
 * same nprogs programs in DEVICE memory.  d_descs (ndescs), d_items, d_counters
 * and d_state (3 int32) are DEVICE memory; every descriptor must pass
 * pgx_check_instance with the programs its items name.  ctas = 0: as many CTAs
 * as fit on the device at once; threads = 0: the largest nthreads of the
 * programs (every program runs with the launch's CTA size). */
typedef struct pgx_persist_item {
  int32_t prog, desc, tile, wait, need, done;
} pgx_persist_item;
#define PGX_PERSIST_TIMEOUT 1
#define PGX_PERSIST_BAD_ITEM 2
int pgx_run_persistent(const pgx_program* h_progs, const pgx_program* d_progs, int32_t nprogs,
                       const pgx_instance* d_descs, int32_t ndescs, const pgx_persist_item* d_items,
                       int32_t nitems, int32_t* d_counters, int32_t ncounters, int32_t* d_state,
                       int32_t ctas, int32_t threads, int64_t spin_limit, void* stream);
/* The launch shape pgx_run_persistent uses for these programs: CTA size, CTAs
 * resident per SM and dynamic shared memory per CTA (bytes). */
int pgx_persistent_shape(const pgx_program* h_progs, int32_t nprogs, int32_t threads, int32_t* out_threads,
                         int32_t* out_ctas_per_sm, int64_t* out_smem);
/* state[1] (0 = the last launch completed every item), synchronising `stream`. */
int pgx_persist_error(const int32_t* d_state, int32_t* error, int32_t* where, void* stream);

/* ------------------------------------------------ reference-facing kernels */

/* DCT-I along `axis` of an n0 x n1 array, in -> out (may alias).
 * mode PGX_DCT_RAW : scipy.fftpack.dctn(f, type=1, axes=(axis,))  (chebyshev.py:85-93)
 * mode PGX_DCT_FWD : Chebyshev.forward_fft incl. solve_mass       (chebyshev.py:67-76,143-149)
 * mode PGX_DCT_BWD : Chebyshev.backward_fft                         (chebyshev.py:78-83)
 * mode PGX_DCT_FWD_T / PGX_DCT_BWD_T : the transposes of FWD / BWD (adjoints for reverse mode)
 * n_in <= n zero-pads the input along axis (pypde zero_pad, bases/utils.py:88-109);
 * n_out <= n truncates the output (zero_unpad, bases/utils.py:112-115). */
int pgx_dct1(const double* in, int64_t in_s0, int64_t in_s1, int32_t n_in,
             double* out, int64_t out_s0, int64_t out_s1, int32_t n_out,
             int32_t n, int32_t nlines, int32_t axis, int32_t mode, void* stream);

/* Two-axis Chebyshev transform of an n0_in x n1_in array: axis 0 with the DCT-I of
 * N0 points, then axis 1 with N1 points (FieldBase.forward / backward over both axes,
 * field.py:14-56).  PGX_DCT_BWD: coefficients zero-padded to N0 x N1 -> values on the
 * (3/2-dealiased) grid; PGX_DCT_FWD: values -> coefficients truncated to
 * n0_out x n1_out after each axis.  `work` is caller-provided device scratch of at
 * least n0_out * n1_in doubles holding the result of the axis-0 pass. */
int pgx_cheb_transform_2d(const double* in, int64_t in_s0, int64_t in_s1, int32_t n0_in, int32_t n1_in,
                          double* out, int64_t out_s0, int64_t out_s1, int32_t n0_out, int32_t n1_out,
                          int32_t N0, int32_t N1, int32_t mode, double* work, int64_t work_doubles,
                          void* stream);

/* Zero-allocation variant of pgx_cheb_transform_2d.  No counterpart in the
 * reference: it serves callers that cannot let a library allocate device memory
 * (host codes that own all device memory through their own pool or budget, and
 * time loops that must not hit the device-wide synchronisation of cudaMalloc /
 * cudaFree).  Same arguments and results as pgx_cheb_transform_2d without `work`;
 * the scratch between the two axis passes (at most PGX_NOALLOC_SCRATCH_DOUBLES =
 * n0_out * n1_in doubles, 16 MiB) and the twiddle tables live in static device
 * arrays that every GPU loading the library holds until exit.  Lengths N0, N1
 * (2 <= N <= PGX_LMAX - 8, as for pgx_cheb_transform_2d) must have n-1 = 2^a 3^b
 * (FFT plans only).  Larger or other sizes return
 * PGX_E_ARG before any launch.  It calls no cudaMalloc, cudaFree or other
 * allocating routine.  The first call on a device looks up the arrays' device
 * addresses (cudaGetSymbolAddress); make that first call before any stream
 * capture.  All calls share the arrays and they keep the last call's contents:
 * calls that overlap on the GPU race (keep them on one stream). */
#define PGX_NOALLOC_SCRATCH_DOUBLES (1 << 21)
int pgx_cheb_transform_2d_noalloc(const double* in, int64_t in_s0, int64_t in_s1, int32_t n0_in, int32_t n1_in,
                                  double* out, int64_t out_s0, int64_t out_s1, int32_t n0_out, int32_t n1_out,
                                  int32_t N0, int32_t N1, int32_t mode, void* stream);

/* Chebyshev derivative recurrence applied `count` times along axis, n points.
 * Replaces differentiate_cheby.diff_1d / diff_2d (differentiate_cheby.f90:1-53,
 * called at chebyshev.py:124,128). */
int pgx_cheb_diff(const double* c, int64_t c_s0, int64_t c_s1,
                  double* dc, int64_t dc_s0, int64_t dc_s1,
                  int32_t n, int32_t nlines, int32_t axis, int32_t count, void* stream);

/* Transpose (adjoint) of pgx_cheb_diff: (D^T)^count along axis.  No reference counterpart:
 * the backward of the derivative for reverse-mode differentiation of the time step. */
int pgx_cheb_diff_t(const double* c, int64_t c_s0, int64_t c_s1,
                    double* dc, int64_t dc_s0, int64_t dc_s1,
                    int32_t n, int32_t nlines, int32_t axis, int32_t count, void* stream);

/* Stencil plans: Galerkin <-> Chebyshev for ChebDirichlet ("CD") / ChebNeumann
 * ("CN") of N points (chebyshev.py:287-337, 382-392, 426-436). */
typedef struct pgx_stencil_plan pgx_stencil_plan;
int pgx_stencil_plan_create(const char* key, int32_t N, pgx_stencil_plan** plan);
int pgx_stencil_plan_destroy(pgx_stencil_plan* plan);
/* u = S v  (to_chebyshev, chebyshev.py:287-293): in has N-2 points, out N. */
int pgx_stencil_to_chebyshev(const pgx_stencil_plan* plan,
                             const double* in, int64_t in_s0, int64_t in_s1,
                             double* out, int64_t out_s0, int64_t out_s1,
                             int32_t nlines, int32_t axis, void* stream);
/* v = (S^T S)^-1 S^T u  (from_chebyshev / _solve_stencil_inv, chebyshev.py:295-329,
 * with the offset-2 TDMA of tdma.f90:56-107): in has N points, out N-2. */
int pgx_stencil_from_chebyshev(const pgx_stencil_plan* plan,
                               const double* in, int64_t in_s0, int64_t in_s1,
                               double* out, int64_t out_s0, int64_t out_s1,
                               int32_t nlines, int32_t axis, void* stream);

/* Transposes of the two stencil maps, for reverse mode (no reference counterpart):
 * S^T (in N points, out N-2) and S (S^T S)^-1 (in N-2 points, out N). */
int pgx_stencil_transpose(const pgx_stencil_plan* plan,
                          const double* in, int64_t in_s0, int64_t in_s1,
                          double* out, int64_t out_s0, int64_t out_s1,
                          int32_t nlines, int32_t axis, void* stream);
int pgx_stencil_from_chebyshev_t(const pgx_stencil_plan* plan,
                                 const double* in, int64_t in_s0, int64_t in_s1,
                                 double* out, int64_t out_s0, int64_t out_s1,
                                 int32_t nlines, int32_t axis, void* stream);

/* Offset-k tridiagonal solve, k = 2 (tdma.solve_tdma_1d/_2d, tdma.f90:2-107,
 * called from tdma.py:92-100).  a (n-2), b (n), c (n-2) are HOST arrays. */
typedef struct pgx_tdma_plan pgx_tdma_plan;
int pgx_tdma_plan_create(const double* a, const double* b, const double* c, int32_t n,
                         int32_t k, pgx_tdma_plan** plan);
int pgx_tdma_plan_destroy(pgx_tdma_plan* plan);
int pgx_tdma_solve(const pgx_tdma_plan* plan, const double* d, int64_t d_s0, int64_t d_s1,
                   double* x, int64_t x_s0, int64_t x_s1, int32_t nlines, int32_t axis,
                   void* stream);

/* Pre-factored four-diagonal (-2, 0, +2, +4) solve, in place along axis.
 * l (n-2), d (n), u1 (n-2), u2 (n-4) are the HOST diagonals after Plan_fdma.FDMA_LU
 * (plans.py:226-234); replaces fdma.solve_fdma_1d / _2d (fdma.f90:1-98, plans.py:211-224). */
typedef struct pgx_fdma_plan pgx_fdma_plan;
int pgx_fdma_plan_create(const double* l, const double* d, const double* u1, const double* u2,
                         int32_t n, pgx_fdma_plan** plan);
int pgx_fdma_plan_destroy(pgx_fdma_plan* plan);
int pgx_fdma_solve(const pgx_fdma_plan* plan, double* x, int64_t s0, int64_t s1,
                   int32_t nlines, int32_t axis, void* stream);

/* Transposed solve A^T x = b with the same plan (adjoint of pgx_fdma_solve), in place. */
int pgx_fdma_solve_t(const pgx_fdma_plan* plan, double* x, int64_t s0, int64_t s1,
                     int32_t nlines, int32_t axis, void* stream);

/* Upper offset-2 bidiagonal back substitution (twodma.solve_twodma_1d/_2d,
 * twodma.f90:2-62, plans.py:160-172): d (n), u (n-2) HOST diagonals; in place. */
int pgx_twodma_plan_create(const double* d, const double* u, int32_t n, pgx_fdma_plan** plan);

/* Fast-diagonalisation Poisson sweep: for every line i, (A + lam_i C) x_i = b_i
 * along axis 0 with the singular rule of fdma.f90:176-179 (|lam_i| < 1e-10 ->
 * solve rows 1: and set x_0 = 0).  A, C (n x n, row-major) and lam (m) are HOST
 * arrays; every per-eigenvalue LU factorisation (init_fdma, fdma.f90:102-143) is
 * done once at plan creation.  Replaces fdma.solve_fdma_type2 (fdma.f90:146-195,
 * plans.py:310-314). */
typedef struct pgx_poisson_plan pgx_poisson_plan;
int pgx_poisson_plan_create(const double* A, const double* C, const double* lam,
                            int32_t n, int32_t m, int32_t singular, pgx_poisson_plan** plan);
int pgx_poisson_plan_destroy(pgx_poisson_plan* plan);
/* axis 0: line j is column j (the reference's call path); axis 1: line j is row j. */
int pgx_poisson_solve(const pgx_poisson_plan* plan, double* x, int64_t s0, int64_t s1,
                      int32_t axis, void* stream);

/* Transposed per-line sweep (adjoint of pgx_poisson_solve), in place. */
int pgx_poisson_solve_t(const pgx_poisson_plan* plan, double* x, int64_t s0, int64_t s1,
                        int32_t axis, void* stream);

/* Matrix applied along an axis, out = A in (MatrixBase.dot, matrix.py:41-56, used by
 * PlanRHS, plans.py:54-74).  A (rows x cols, row-major HOST) is stored banded when
 * its nonzeros lie on diagonals offset0 + 2j (the pseudo-inverse B and B S of
 * dmsuite.py:327-368), dense otherwise (the Poisson H_y, Q_y of poisson.py:93-96). */
typedef struct pgx_matrix_plan pgx_matrix_plan;
int pgx_matrix_plan_create(const double* A, int32_t rows, int32_t cols, pgx_matrix_plan** plan);
int pgx_matrix_plan_destroy(pgx_matrix_plan* plan);
int pgx_matrix_apply(const pgx_matrix_plan* plan, const double* in, int64_t in_s0, int64_t in_s1,
                     double* out, int64_t out_s0, int64_t out_s1, int32_t nlines, int32_t axis,
                     void* stream);
/* 1 if the plan is stored banded, 0 if dense. */
int pgx_matrix_plan_is_banded(const pgx_matrix_plan* plan);

/* Device tables for line programs built by the host: twiddle factors of the
 * DCT-I of n points (2(n-1) complex values exp(-2 pi i k / (2(n-1))), then the
 * n-1 doubles 0.5 + Im(tw[m]) = 1/2 - sin(pi m / (n-1)) of the folded transform),
 * and the stencil sub-diagonal table.  The returned device
 * pointer is owned by the library and valid until process exit. */
int pgx_dct_table(int32_t n, const double** table);

/* ------------------------------------------------------------ measurement
 * No counterpart in the reference: the FP64 roofline denominator.  Launches
 * `ctas` x `threads` threads that each run 8 independent FMA chains of `iters`
 * steps and store one double (out: ctas * threads doubles of device memory);
 * the caller times it with events on `stream`.  pgx_fp64_fma_probe_flops gives
 * the flops of one launch (an FMA counts two). */
int pgx_fp64_fma_probe(double* out, int32_t ctas, int32_t threads, int32_t iters, void* stream);
int64_t pgx_fp64_fma_probe_flops(int32_t ctas, int32_t threads, int32_t iters);

#ifdef __cplusplus
}
#endif
#endif /* PGX_H */
