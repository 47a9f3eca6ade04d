// C ABI of libpypde_gb300.so: validation, launches, operator plans.
//
// Host-side factorisations (banded LU, offset-2 TDMA, per-eigenvalue Poisson
// factors) happen once per plan in FP64 on the CPU; the device only ever
// multiplies by stored reciprocals.

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "pgx.h"

namespace pgx {
int launch_single(const pgx_program* P, const pgx_instance* I, cudaStream_t s, int ntiles);
int launch_batched(const pgx_program* P, const pgx_instance* d_insts, const int32_t* d_work, int nwork,
                   cudaStream_t s);
int persistent_shape(const pgx_program* progs, int nprogs, int threads, int* out_threads, int* ctas_per_sm,
                     int64_t* smem);
int launch_persistent(const pgx_program* d_progs, int nprogs, const pgx_instance* d_descs, int ndescs,
                      const pgx_persist_item* d_items, int nitems, int32_t* d_counters, int ncounters,
                      int32_t* d_state, int ctas, int threads, int64_t smem, long long spin_limit, cudaStream_t s);
}

static thread_local int g_last_cuda = 0;

static int cuda_fail(cudaError_t e) {
  g_last_cuda = (int)e;
  return PGX_E_CUDA;
}
#define PGX_CUDA(call)                          \
  do {                                          \
    cudaError_t e_ = (call);                    \
    if (e_ != cudaSuccess) return cuda_fail(e_); \
  } while (0)

extern "C" const char* pgx_error_string(int code) {
  switch (code) {
    case PGX_OK: return "ok";
    case PGX_E_ARG: return "invalid argument (shape, stride, length or enum)";
    case PGX_E_CUDA: return "CUDA runtime error (see pgx_last_cuda_error)";
    case PGX_E_SMEM: return "tile does not fit in shared memory";
    case PGX_E_PLAN: return "null plan handle";
    case PGX_E_SINGULAR: return "zero pivot in banded factorisation";
    default: return "unknown pgx error";
  }
}
extern "C" int pgx_last_cuda_error(void) { return g_last_cuda; }
extern "C" int pgx_version(void) { return 1; }

static int smem_optin_max() {
  static int v = 0;
  if (!v) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (v <= 0) v = 48 * 1024;
  }
  return v;
}

// Longest DCT length run as a dense contraction on the FP64 tensor cores (and the longest
// dense operator for which DMMA beats FMA chains on GB300, whose FP64 tensor rate is below
// its DFMA rate).
static const int DENSE_MMA_MAX_N = 33;

// The program's own consistency (limits, slots, indices); the shared-memory capacity is checked
// against the device by check_program.
static int check_program_shape(const pgx_program* P) {
  if (!P) return PGX_E_ARG;
  if (P->axis < 0 || P->axis > 1 || P->tb < 1 || P->lcap < 1 || P->lcap > PGX_LMAX + 8) return PGX_E_ARG;
  if (P->nslots < 1 || P->nslots > PGX_MAX_SLOTS || P->nops < 0 || P->nops > PGX_MAX_OPS) return PGX_E_ARG;
  if (P->nthreads < 32 || P->nthreads > PGX_MAX_THREADS || (P->nthreads & 31)) return PGX_E_ARG;
  bool has_dct = false;
  for (int o = 0; o < P->nops; ++o) has_dct |= P->ops[o].code == PGX_OP_DCT;
  // DCT ops need the FFT buffers (fft_n) and run in the kernel build for up to 768 threads
  if (has_dct && (P->fft_n < 2 || P->nthreads > PGX_MAX_THREADS_FFT)) return PGX_E_ARG;
  if (P->lines_len < 0 || P->lines_len >= PGX_MAX_LEN) return PGX_E_ARG;
  if (P->fft_n > P->lcap) return PGX_E_ARG;
  for (int o = 0; o < P->nops; ++o) {
    const pgx_op& op = P->ops[o];
    if (op.a < 0 || op.a >= P->nslots) return PGX_E_ARG;
    const bool uses_b = op.code == PGX_OP_AXPY || op.code == PGX_OP_MUL || op.code == PGX_OP_COPY;
    if (uses_b && (op.b < 0 || op.b >= P->nslots)) return PGX_E_ARG;
    const bool chain = op.code == PGX_OP_DIFF || op.code == PGX_OP_DIFF_T || op.code == PGX_OP_TDMA2 ||
                       op.code == PGX_OP_FDMA || op.code == PGX_OP_FDMA_T;
    if ((chain || op.code == PGX_OP_DCT) && op.a + (op.b > 1 ? op.b : 1) > P->nslots) return PGX_E_ARG;
    // a DCT in the slot's own lines: one slot, line pairs filling the tile
    if (op.code == PGX_OP_DCT && (op.k & PGX_DCT_SLOT) && (op.b > 1 || (P->tb & 1))) return PGX_E_ARG;
    if (chain && (op.code == PGX_OP_FDMA || op.code == PGX_OP_FDMA_T) && op.mat + (op.b > 1 ? op.b : 1) > PGX_MAX_MAT)
      return PGX_E_ARG;
    if (op.arr >= PGX_MAX_ARR || op.mat >= PGX_MAX_MAT || op.len >= PGX_MAX_LEN || op.par >= PGX_MAX_PAR) return PGX_E_ARG;
  }
  return PGX_OK;
}

static int check_program(const pgx_program* P) {
  int rc = check_program_shape(P);
  if (rc) return rc;
  int64_t need = pgx_program_smem(P) + 1024;
  if (need > smem_optin_max()) return PGX_E_SMEM;
  return PGX_OK;
}

// Checks the op arguments of a single instance against its lengths and arrays.
static int check_instance(const pgx_program* P, const pgx_instance* I) {
  int nl = I->len[P->lines_len];
  if (nl < 0) return PGX_E_ARG;
  for (int o = 0; o < P->nops; ++o) {
    const pgx_op& op = P->ops[o];
    switch (op.code) {
      case PGX_OP_LOAD:
      case PGX_OP_SETLEN:
        if (op.len < 0 || I->len[op.len] < 0 || I->len[op.len] > P->lcap - 1) return PGX_E_ARG;
        if (op.code == PGX_OP_SETLEN) break;
        /* fallthrough */
      case PGX_OP_LOAD_ADD:
      case PGX_OP_LOAD_MUL:
      case PGX_OP_STORE:
      case PGX_OP_STORE_ADD: {
        if (op.arr < 0) return PGX_E_ARG;
        const pgx_array& a = I->arr[op.arr];
        if (!a.ptr && (a.n0 > 0 && a.n1 > 0)) return PGX_E_ARG;
        int ne = P->axis == 0 ? a.n0 : a.n1;
        if (ne > P->lcap - 1) return PGX_E_ARG;
        break;
      }
      case PGX_OP_DENSE:
      case PGX_OP_BANDED:
        if (op.mat < 0 || !I->mat[op.mat] || op.len < 0 || I->len[op.len] > P->lcap - 1) return PGX_E_ARG;
        break;
      case PGX_OP_STENCIL:
      case PGX_OP_STENCIL_T:
      case PGX_OP_TDMA2:
      case PGX_OP_FDMA:
      case PGX_OP_POISSON:
      case PGX_OP_FDMA_T:
      case PGX_OP_POISSON_T:
      case PGX_OP_DCT:
        if (op.mat < 0 || !I->mat[op.mat]) return PGX_E_ARG;
        break;
      default: break;
    }
  }
  return PGX_OK;
}

extern "C" int pgx_run(const pgx_program* P, const pgx_instance* I, void* stream) {
  int rc = check_program(P);
  if (rc) return rc;
  if (!I) return PGX_E_ARG;
  rc = check_instance(P, I);
  if (rc) return rc;
  int nl = I->len[P->lines_len];
  if (nl == 0) return PGX_OK;
  int ntiles = (nl + P->tb - 1) / P->tb;
  int e = pgx::launch_single(P, I, (cudaStream_t)stream, ntiles);
  if (e) return cuda_fail((cudaError_t)e);
  return PGX_OK;
}

extern "C" int pgx_check_instance(const pgx_program* P, const pgx_instance* I) {
  int rc = check_program_shape(P);
  if (rc) return rc;
  if (!I || P->lines_len < 0) return PGX_E_ARG;
  return check_instance(P, I);
}

extern "C" int pgx_run_batched(const pgx_program* P, const pgx_instance* d_insts, const int32_t* d_work,
                               int32_t nwork, void* stream) {
  int rc = check_program(P);
  if (rc) return rc;
  if (nwork < 0 || (nwork > 0 && (!d_insts || !d_work))) return PGX_E_ARG;
  if (pgx_program_smem(P) + (int64_t)sizeof(pgx_instance) + 1024 > smem_optin_max()) return PGX_E_SMEM;
  if (nwork == 0) return PGX_OK;
  int e = pgx::launch_batched(P, d_insts, d_work, nwork, (cudaStream_t)stream);
  if (e) return cuda_fail((cudaError_t)e);
  return PGX_OK;
}

// --------------------------------------------------------- persistent steps
extern "C" int pgx_persistent_shape(const pgx_program* h_progs, int32_t nprogs, int32_t threads, int32_t* out_threads,
                                    int32_t* out_ctas_per_sm, int64_t* out_smem) {
  if (!h_progs || nprogs < 1 || threads < 0 || threads > PGX_MAX_THREADS_FFT || (threads & 31) || !out_threads ||
      !out_ctas_per_sm || !out_smem)
    return PGX_E_ARG;
  for (int i = 0; i < nprogs; ++i) {
    int rc = check_program_shape(h_progs + i);
    if (rc) return rc;
  }
  int nt = 0, per = 0;
  int64_t smem = 0;
  int e = pgx::persistent_shape(h_progs, nprogs, threads, &nt, &per, &smem);
  if (e) return cuda_fail((cudaError_t)e);
  if (nt > PGX_MAX_THREADS_FFT || smem > smem_optin_max()) return PGX_E_SMEM;
  *out_threads = nt;
  *out_ctas_per_sm = per;
  *out_smem = smem;
  return PGX_OK;
}

extern "C" int pgx_run_persistent(const pgx_program* h_progs, const pgx_program* d_progs, int32_t nprogs,
                                  const pgx_instance* d_descs, int32_t ndescs, const pgx_persist_item* d_items,
                                  int32_t nitems, int32_t* d_counters, int32_t ncounters, int32_t* d_state,
                                  int32_t ctas, int32_t threads, int64_t spin_limit, void* stream) {
  if (!d_progs || !d_descs || ndescs < 1 || nitems < 0 || (nitems > 0 && !d_items) || !d_counters || ncounters < 1 ||
      !d_state || ctas < 0 || spin_limit < 1)
    return PGX_E_ARG;
  int nt = 0, per = 0;
  int64_t smem = 0;
  int rc = pgx_persistent_shape(h_progs, nprogs, threads, &nt, &per, &smem);
  if (rc) return rc;
  if (per < 1) return PGX_E_SMEM;
  int dev = 0, sms = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (ce != cudaSuccess) return cuda_fail(ce);
  const int grid = ctas > 0 ? ctas : per * sms;
  int e = pgx::launch_persistent(d_progs, nprogs, d_descs, ndescs, d_items, nitems, d_counters, ncounters, d_state,
                                 grid, nt, smem, (long long)spin_limit, (cudaStream_t)stream);
  if (e) return cuda_fail((cudaError_t)e);
  return PGX_OK;
}

extern "C" int pgx_persist_error(const int32_t* d_state, int32_t* error, int32_t* where, void* stream) {
  if (!d_state || !error) return PGX_E_ARG;
  int32_t h[3] = {0, 0, 0};
  cudaError_t e = cudaMemcpyAsync(h, d_state, sizeof(h), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e);
  *error = h[1];
  if (where) *where = h[2];
  return PGX_OK;
}

// ------------------------------------------------------------ device tables
namespace {
std::mutex g_mu;

int upload(const std::vector<double>& h, double** d) {
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, h.size() * sizeof(double) + 16);
  if (e != cudaSuccess) return cuda_fail(e);
  e = cudaMemcpy(p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(p);
    return cuda_fail(e);
  }
  *d = (double*)p;
  return PGX_OK;
}

bool fft_length_ok(int L) {
  if (L < 2) return false;
  while (L % 2 == 0) L /= 2;
  while (L % 3 == 0) L /= 3;
  return L == 1;
}

// key (device, n) -> twiddles exp(-2 pi i k / L), L = 2(n-1), and the fold coefficients
std::map<std::pair<int, int>, double*> g_tw;
// key (device, n, mode) -> dense scaled cosine matrix for lengths the FFT does not cover
std::map<std::pair<int, int>, double*> g_dense;

int device_id() {
  int d = 0;
  cudaGetDevice(&d);
  return d;
}

int twiddles(int n, const double** out) {
  int L = 2 * (n - 1);
  if (!fft_length_ok(L)) return PGX_E_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  auto key = std::make_pair(device_id(), n);
  auto it = g_tw.find(key);
  if (it != g_tw.end()) {
    *out = it->second;
    return PGX_OK;
  }
  // L complex twiddles, then the fold coefficients 1/2 - sin(pi m / N) (m < N = L/2), each the
  // FP64 sum 0.5 + Im(tw[m]) that the kernels would otherwise form per point
  std::vector<double> h(2 * (size_t)L + L / 2);
  const double pi = 3.14159265358979323846;
  for (int k = 0; k < L; ++k) {
    double a = 2.0 * pi * (double)k / (double)L;
    h[2 * k] = cos(a);
    h[2 * k + 1] = -sin(a);
  }
  // exact values on the axes
  for (int k = 0; k < L; ++k) {
    if ((4 * k) % L == 0) {
      int q = (4 * k) / L;
      const double cs[4] = {1, 0, -1, 0}, sn[4] = {0, 1, 0, -1};
      h[2 * k] = cs[q];
      h[2 * k + 1] = -sn[q];
    }
  }
  for (int m = 0; m < L / 2; ++m) h[2 * (size_t)L + m] = 0.5 + h[2 * m + 1];
  double* d = nullptr;
  int rc = upload(h, &d);
  if (rc) return rc;
  g_tw[key] = d;
  *out = d;
  return PGX_OK;
}

// Host copies of the per-mode diagonal scalings of the kernels (y = post C (pre x)).
double dct_pre_h(int mode, int j, int N) {
  const bool end = (j == 0 || j == N);
  const double sg = (j & 1) ? -1.0 : 1.0;
  switch (mode) {
    case PGX_DCT_BWD: return end ? sg : 0.5 * sg;
    case PGX_DCT_FWD_T: return sg * (0.5 / N);
    case PGX_DCT_BWD_T: return end ? 1.0 : 0.5;
    default: return 1.0;
  }
}
double dct_post_h(int mode, int k, int N) {
  const bool end = (k == 0 || k == N);
  const double sg = (k & 1) ? -1.0 : 1.0;
  switch (mode) {
    case PGX_DCT_FWD: return sg * (end ? 0.5 / N : 1.0 / N);
    case PGX_DCT_FWD_T: return end ? 1.0 : 2.0;
    case PGX_DCT_BWD_T: return sg;
    default: return 1.0;
  }
}

// DCT-I as a dense matrix with the Chebyshev pre/post scaling folded in.
int dense_dct(int n, int mode, const double** out) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto key = std::make_pair(device_id(), n * 8 + mode);
  auto it = g_dense.find(key);
  if (it != g_dense.end()) {
    *out = it->second;
    return PGX_OK;
  }
  const int N = n - 1;
  const double pi = 3.14159265358979323846;
  std::vector<double> h((size_t)n * n);
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j) {
      double c;
      if (j == 0) c = 1.0;
      else if (j == N) c = (k & 1) ? -1.0 : 1.0;
      else {
        long long r = ((long long)j * k) % (2 * N);  // cos(pi j k / N) with exact argument reduction
        c = 2.0 * cos(pi * (double)r / (double)N);
      }
      h[(size_t)k * n + j] = dct_post_h(mode, k, N) * c * dct_pre_h(mode, j, N);
    }
  double* d = nullptr;
  int rc = upload(h, &d);
  if (rc) return rc;
  g_dense[key] = d;
  *out = d;
  return PGX_OK;
}

int round_odd(int x) { return x | 1; }

// Lines per CTA and CTA size for a single-instance pass.
void pick_tile(pgx_program* P, int nlines, int maxlen, int nbuf, int fft_n) {
  P->lcap = round_odd(maxlen + 1);
  // FFT buffers: 2 buffers x stride complex per line pair (see pgx_fft_stride)
  int64_t stride = fft_n > 1 ? (((fft_n - 1) & 1) == 0 ? fft_n - 1 : 2 * (fft_n - 1)) : 0;
  int64_t per_line = (int64_t)8 * nbuf * P->lcap + 16 * stride + 8;
  int64_t budget = smem_optin_max() - 4096;
  int tbmax = (int)(budget / per_line);
  if (tbmax < 1) tbmax = 1;
  int tb = (nlines + 151) / 152;
  if (fft_n > 1 && tb < 2) tb = 2;
  if (tb > 32) tb = 32;
  if (tb > tbmax) tb = tbmax;
  if (tb < 1) tb = 1;
  P->tb = tb;
  int work = tb * P->lcap / 2;
  int nt = ((work + 31) / 32) * 32;
  if (nt < 64) nt = 64;
  if (nt > 512) nt = 512;
  P->nthreads = nt;
  // Sequential chain sweeps with few lines in the launch (fewer chains than ~64 per SM)
  // run one warp per (line, parity) chain with a warp-parallel scan.
  bool chains = false;
  for (int o = 0; o < P->nops; ++o) {
    const int code = P->ops[o].code;
    chains |= code == PGX_OP_TDMA2 || code == PGX_OP_FDMA || code == PGX_OP_FDMA_T || code == PGX_OP_POISSON ||
              code == PGX_OP_POISSON_T;
  }
  if (chains && 2 * (int64_t)nlines < 152 * 64) {
    for (int o = 0; o < P->nops; ++o) {
      pgx_op& op = P->ops[o];
      if (op.code == PGX_OP_TDMA2 || op.code == PGX_OP_FDMA || op.code == PGX_OP_FDMA_T ||
          op.code == PGX_OP_POISSON || op.code == PGX_OP_POISSON_T)
        op.k = (int16_t)(op.k | PGX_CHAIN_WARP);
    }
    int wt = 64 * tb;  // two chains (parities) per line, one warp each
    P->nthreads = wt < 256 ? 256 : (wt > PGX_MAX_THREADS ? PGX_MAX_THREADS : wt);
  }
}

pgx_op mk(int code, int a, int b = -1, int arr = -1, int mat = -1, int len = -1, int k = 0, double alpha = 1.0) {
  pgx_op op;
  op.code = (int16_t)code; op.a = (int16_t)a; op.b = (int16_t)b; op.arr = (int16_t)arr;
  op.mat = (int16_t)mat; op.len = (int16_t)len; op.par = -1; op.k = (int16_t)k; op.alpha = alpha;
  return op;
}

void set_arr(pgx_instance& I, int idx, const double* p, int64_t s0, int64_t s1, int n0, int n1) {
  I.arr[idx].ptr = const_cast<double*>(p);
  I.arr[idx].s0 = s0; I.arr[idx].s1 = s1; I.arr[idx].n0 = n0; I.arr[idx].n1 = n1;
}

// Array view (n_axis elements along `axis`, nlines lines) from pointer + strides.
void set_axis_arr(pgx_instance& I, int idx, const double* p, int64_t s0, int64_t s1, int axis, int nel, int nlines) {
  if (axis == 0) set_arr(I, idx, p, s0, s1, nel, nlines);
  else set_arr(I, idx, p, s0, s1, nlines, nel);
}

void init_prog(pgx_program& P, pgx_instance& I, int axis) {
  memset(&P, 0, sizeof(P));
  memset(&I, 0, sizeof(I));
  P.axis = axis;
  P.lines_len = 0;
  P.nslots = 1;
}
}  // namespace

extern "C" int pgx_dct_table(int32_t n, const double** table) {
  if (!table || n < 2 || n > PGX_LMAX - 8) return PGX_E_ARG;
  return twiddles(n, table);
}

// ------------------------------------------------------------------- DCT-I
// One DCT-I pass along `axis`: `in` (n_in points along axis, zero-padded to n)
// -> `out` (first n_out points).  `tab` is the twiddle table (fft) or the dense
// scaled cosine matrix.
int pgx_dct_pass(const double* in, int64_t in_s0, int64_t in_s1, int32_t n_in, double* out, int64_t out_s0,
                 int64_t out_s1, int32_t n_out, int32_t n, int32_t nlines, int32_t axis, int32_t mode,
                 const double* tab, bool fft, void* stream) {
  pgx_program P;
  pgx_instance I;
  init_prog(P, I, axis);
  I.len[0] = nlines;
  I.len[1] = n;
  set_axis_arr(I, 0, in, in_s0, in_s1, axis, n_in, nlines);
  set_axis_arr(I, 1, out, out_s0, out_s1, axis, n_out, nlines);
  I.mat[0] = tab;
  P.nops = 3;
  P.ops[0] = mk(PGX_OP_LOAD, 0, -1, 0, -1, 1);
  const bool mma = !fft && n <= DENSE_MMA_MAX_N;
  if (fft) {
    P.ops[1] = mk(PGX_OP_DCT, 0, -1, -1, 0, -1, mode);
    P.fft_n = n;
  } else {
    P.ops[1] = mk(PGX_OP_DENSE, 0, -1, -1, 0, 1, mma ? PGX_DENSE_MMA : 0);
  }
  P.ops[2] = mk(PGX_OP_STORE, 0, -1, 1);
  pick_tile(&P, nlines, n, 2, P.fft_n);
  if (mma) {  // one 8-line tensor-core tile per CTA, a warp per 8-row block
    P.tb = 8;
    P.nthreads = 32 * ((n + 7) / 8);
  }
  return pgx_run(&P, &I, stream);
}

bool pgx_fft_length_ok(int n) { return fft_length_ok(2 * (n - 1)); }

// FFT or dense matrix for a DCT pass of `nlines` lines of length n.  Measured on GB300
// (fwd + bwd along one axis of an N x N field): the dense contraction on the FP64 tensor
// cores beats the FFT at N = 33 (latency: two phases instead of nine) and loses from N = 65
// on (1.7x at 65, 18x at 1025); for many lines the FFT's 3-4x fewer FP64 operations win.
static bool dct_use_fft(int n, int nlines) {
  if (!fft_length_ok(2 * (n - 1))) return false;
  return !(n <= DENSE_MMA_MAX_N && nlines <= 8 * 152);
}

extern "C" int pgx_dct1(const double* in, int64_t in_s0, int64_t in_s1, int32_t n_in, double* out, int64_t out_s0,
                        int64_t out_s1, int32_t n_out, int32_t n, int32_t nlines, int32_t axis, int32_t mode,
                        void* stream) {
  if (!in || !out || n < 2 || n > PGX_LMAX - 8 || n_in < 0 || n_in > n || n_out < 0 || n_out > n || nlines < 0 ||
      axis < 0 || axis > 1 || mode < 0 || mode > 4)
    return PGX_E_ARG;
  const double* tab = nullptr;
  bool fft = dct_use_fft(n, nlines);
  int rc = fft ? twiddles(n, &tab) : dense_dct(n, mode, &tab);
  if (rc) return rc;
  return pgx_dct_pass(in, in_s0, in_s1, n_in, out, out_s0, out_s1, n_out, n, nlines, axis, mode, tab, fft, stream);
}

// Both axes: axis 0 (in -> work, n0_out x n1_in, row-major) then axis 1 (work -> out).
extern "C" int pgx_cheb_transform_2d(const double* in, int64_t in_s0, int64_t in_s1, int32_t n0_in, int32_t n1_in,
                                     double* out, int64_t out_s0, int64_t out_s1, int32_t n0_out, int32_t n1_out,
                                     int32_t N0, int32_t N1, int32_t mode, double* work, int64_t work_doubles,
                                     void* stream) {
  if (!in || !out || !work || mode < 0 || mode > 2 || N0 < 2 || N1 < 2 || N0 > PGX_LMAX - 8 || N1 > PGX_LMAX - 8 ||
      n0_in < 0 || n0_in > N0 || n1_in < 0 || n1_in > N1 || n0_out < 0 || n0_out > N0 || n1_out < 0 || n1_out > N1)
    return PGX_E_ARG;
  if (work_doubles < (int64_t)n0_out * n1_in) return PGX_E_ARG;
  const double* t0 = nullptr;
  const double* t1 = nullptr;
  bool f0 = dct_use_fft(N0, n1_in), f1 = dct_use_fft(N1, n0_out);
  int rc = f0 ? twiddles(N0, &t0) : dense_dct(N0, mode, &t0);
  if (!rc) rc = f1 ? twiddles(N1, &t1) : dense_dct(N1, mode, &t1);
  if (rc) return rc;
  rc = pgx_dct_pass(in, in_s0, in_s1, n0_in, work, n1_in, 1, n0_out, N0, n1_in, 0, mode, t0, f0, stream);
  if (rc) return rc;
  return pgx_dct_pass(work, n1_in, 1, n1_in, out, out_s0, out_s1, n1_out, N1, n0_out, 1, mode, t1, f1, stream);
}

// ------------------------------------------------------- derivative recurrence
static int cheb_diff_op(int code, const double* c, int64_t c_s0, int64_t c_s1, double* dc, int64_t dc_s0,
                        int64_t dc_s1, int32_t n, int32_t nlines, int32_t axis, int32_t count, void* stream);

extern "C" int pgx_cheb_diff(const double* c, int64_t c_s0, int64_t c_s1, double* dc, int64_t dc_s0, int64_t dc_s1,
                             int32_t n, int32_t nlines, int32_t axis, int32_t count, void* stream) {
  return cheb_diff_op(PGX_OP_DIFF, c, c_s0, c_s1, dc, dc_s0, dc_s1, n, nlines, axis, count, stream);
}

extern "C" int pgx_cheb_diff_t(const double* c, int64_t c_s0, int64_t c_s1, double* dc, int64_t dc_s0, int64_t dc_s1,
                               int32_t n, int32_t nlines, int32_t axis, int32_t count, void* stream) {
  return cheb_diff_op(PGX_OP_DIFF_T, c, c_s0, c_s1, dc, dc_s0, dc_s1, n, nlines, axis, count, stream);
}

static int cheb_diff_op(int code, const double* c, int64_t c_s0, int64_t c_s1, double* dc, int64_t dc_s0,
                        int64_t dc_s1, int32_t n, int32_t nlines, int32_t axis, int32_t count, void* stream) {
  if (!c || !dc || n < 3 || n > PGX_LMAX - 8 || nlines < 0 || axis < 0 || axis > 1 || count < 0) return PGX_E_ARG;
  pgx_program P;
  pgx_instance I;
  init_prog(P, I, axis);
  I.len[0] = nlines;
  I.len[1] = n;
  set_axis_arr(I, 0, c, c_s0, c_s1, axis, n, nlines);
  set_axis_arr(I, 1, dc, dc_s0, dc_s1, axis, n, nlines);
  P.nops = 3;
  P.ops[0] = mk(PGX_OP_LOAD, 0, -1, 0, -1, 1);
  P.ops[1] = mk(code, 0, -1, -1, -1, -1, count);
  P.ops[2] = mk(PGX_OP_STORE, 0, -1, 1);
  pick_tile(&P, nlines, n, 2, 0);
  return pgx_run(&P, &I, stream);
}

// ---------------------------------------------------------------- stencils
struct pgx_stencil_plan {
  int N;
  double* sub;    // S[i+2, i], i < N-2 (length N)
  double* tdma;   // offset-2 TDMA factors, interleaved (a r, r, w) per index (r: reciprocal pivot)
};
struct pgx_tdma_plan {
  int n;
  double* tab;
};

// Offset-2 TDMA table from diagonals a (n-2, offset -2), b (n), c (n-2, offset +2),
// interleaved per index i: (a_{i-2} r_i, r_i, w_i) with the reciprocal pivot
// r_i = 1/(b_i - a_{i-2} w_{i-2}); the forward sweep g_i = r_i x_i - (a_{i-2} r_i) g_{i-2}
// then has one dependent FMA per step.
static int tdma_table(const double* a, const double* b, const double* c, int n, std::vector<double>& tab) {
  tab.assign(3 * (size_t)n, 0.0);
  std::vector<double> w(n, 0.0);
  for (int i = 0; i < n; ++i) {
    double den = i < 2 ? b[i] : b[i] - a[i - 2] * w[i - 2];
    if (den == 0.0) return PGX_E_SINGULAR;
    if (i < n - 2) w[i] = c[i] / den;
    tab[3 * i] = i < 2 ? 0.0 : a[i - 2] / den;
    tab[3 * i + 1] = 1.0 / den;
    tab[3 * i + 2] = w[i];
  }
  return PGX_OK;
}

extern "C" int pgx_stencil_plan_create(const char* key, int32_t N, pgx_stencil_plan** plan) {
  if (!key || !plan || N < 5 || N > PGX_LMAX - 8) return PGX_E_ARG;
  int kind;
  if (!strcmp(key, "CD") || !strcmp(key, "ChebDirichlet")) kind = 0;
  else if (!strcmp(key, "CN") || !strcmp(key, "ChebNeumann")) kind = 1;
  else return PGX_E_ARG;
  const int M = N - 2;
  std::vector<double> sub(N, 0.0);
  for (int i = 0; i < M; ++i) sub[i] = kind == 0 ? -1.0 : -((double)i / (i + 2)) * ((double)i / (i + 2));
  // S^T S diagonals: d_i = 1 + s_i^2, off_{i,i+2} = s_i (S^T S is symmetric)
  std::vector<double> a(M, 0.0), b(M, 0.0), c(M, 0.0);
  for (int i = 0; i < M; ++i) b[i] = 1.0 + sub[i] * sub[i];
  for (int i = 0; i + 2 < M; ++i) {
    c[i] = sub[i];
    a[i] = sub[i];
  }
  std::vector<double> tab;
  int rc = tdma_table(a.data(), b.data(), c.data(), M, tab);
  if (rc) return rc;
  pgx_stencil_plan* p = new pgx_stencil_plan();
  p->N = N;
  rc = upload(sub, &p->sub);
  if (!rc) rc = upload(tab, &p->tdma);
  if (rc) {
    delete p;
    return rc;
  }
  *plan = p;
  return PGX_OK;
}

extern "C" int pgx_stencil_plan_destroy(pgx_stencil_plan* p) {
  if (!p) return PGX_E_PLAN;
  cudaFree(p->sub);
  cudaFree(p->tdma);
  delete p;
  return PGX_OK;
}

extern "C" int pgx_stencil_to_chebyshev(const pgx_stencil_plan* p, const double* in, int64_t in_s0, int64_t in_s1,
                                        double* out, int64_t out_s0, int64_t out_s1, int32_t nlines, int32_t axis,
                                        void* stream) {
  if (!p) return PGX_E_PLAN;
  if (!in || !out || nlines < 0 || axis < 0 || axis > 1) return PGX_E_ARG;
  pgx_program P;
  pgx_instance I;
  init_prog(P, I, axis);
  I.len[0] = nlines;
  I.len[1] = p->N - 2;
  set_axis_arr(I, 0, in, in_s0, in_s1, axis, p->N - 2, nlines);
  set_axis_arr(I, 1, out, out_s0, out_s1, axis, p->N, nlines);
  I.mat[0] = p->sub;
  P.nops = 3;
  P.ops[0] = mk(PGX_OP_LOAD, 0, -1, 0, -1, 1);
  P.ops[1] = mk(PGX_OP_STENCIL, 0, -1, -1, 0);
  P.ops[2] = mk(PGX_OP_STORE, 0, -1, 1);
  pick_tile(&P, nlines, p->N, 2, 0);
  return pgx_run(&P, &I, stream);
}

extern "C" int pgx_stencil_from_chebyshev(const pgx_stencil_plan* p, const double* in, int64_t in_s0, int64_t in_s1,
                                          double* out, int64_t out_s0, int64_t out_s1, int32_t nlines, int32_t axis,
                                          void* stream) {
  if (!p) return PGX_E_PLAN;
  if (!in || !out || nlines < 0 || axis < 0 || axis > 1) return PGX_E_ARG;
  pgx_program P;
  pgx_instance I;
  init_prog(P, I, axis);
  I.len[0] = nlines;
  I.len[1] = p->N;
  set_axis_arr(I, 0, in, in_s0, in_s1, axis, p->N, nlines);
  set_axis_arr(I, 1, out, out_s0, out_s1, axis, p->N - 2, nlines);
  I.mat[0] = p->sub;
  I.mat[1] = p->tdma;
  P.nops = 4;
  P.ops[0] = mk(PGX_OP_LOAD, 0, -1, 0, -1, 1);
  P.ops[1] = mk(PGX_OP_STENCIL_T, 0, -1, -1, 0);
  P.ops[2] = mk(PGX_OP_TDMA2, 0, -1, -1, 1);
  P.ops[3] = mk(PGX_OP_STORE, 0, -1, 1);
  pick_tile(&P, nlines, p->N, 2, 0);
  return pgx_run(&P, &I, stream);
}

// Transposes of the two stencil maps (adjoints for reverse mode):
//   S^T: N -> N-2 points;  S (S^T S)^-1 (the transpose of from_chebyshev): N-2 -> N points.
extern "C" int pgx_stencil_transpose(const pgx_stencil_plan* p, const double* in, int64_t in_s0, int64_t in_s1,
                                     double* out, int64_t out_s0, int64_t out_s1, int32_t nlines, int32_t axis,
                                     void* stream) {
  if (!p) return PGX_E_PLAN;
  if (!in || !out || nlines < 0 || axis < 0 || axis > 1) return PGX_E_ARG;
  pgx_program P;
  pgx_instance I;
  init_prog(P, I, axis);
  I.len[0] = nlines;
  I.len[1] = p->N;
  set_axis_arr(I, 0, in, in_s0, in_s1, axis, p->N, nlines);
  set_axis_arr(I, 1, out, out_s0, out_s1, axis, p->N - 2, nlines);
  I.mat[0] = p->sub;
  P.nops = 3;
  P.ops[0] = mk(PGX_OP_LOAD, 0, -1, 0, -1, 1);
  P.ops[1] = mk(PGX_OP_STENCIL_T, 0, -1, -1, 0);
  P.ops[2] = mk(PGX_OP_STORE, 0, -1, 1);
  pick_tile(&P, nlines, p->N, 2, 0);
  return pgx_run(&P, &I, stream);
}

extern "C" int pgx_stencil_from_chebyshev_t(const pgx_stencil_plan* p, const double* in, int64_t in_s0,
                                            int64_t in_s1, double* out, int64_t out_s0, int64_t out_s1,
                                            int32_t nlines, int32_t axis, void* stream) {
  if (!p) return PGX_E_PLAN;
  if (!in || !out || nlines < 0 || axis < 0 || axis > 1) return PGX_E_ARG;
  pgx_program P;
  pgx_instance I;
  init_prog(P, I, axis);
  I.len[0] = nlines;
  I.len[1] = p->N - 2;
  set_axis_arr(I, 0, in, in_s0, in_s1, axis, p->N - 2, nlines);
  set_axis_arr(I, 1, out, out_s0, out_s1, axis, p->N, nlines);
  I.mat[0] = p->sub;
  I.mat[1] = p->tdma;
  P.nops = 4;
  P.ops[0] = mk(PGX_OP_LOAD, 0, -1, 0, -1, 1);
  P.ops[1] = mk(PGX_OP_TDMA2, 0, -1, -1, 1);
  P.ops[2] = mk(PGX_OP_STENCIL, 0, -1, -1, 0);
  P.ops[3] = mk(PGX_OP_STORE, 0, -1, 1);
  pick_tile(&P, nlines, p->N, 2, 0);
  return pgx_run(&P, &I, stream);
}

extern "C" int pgx_tdma_plan_create(const double* a, const double* b, const double* c, int32_t n, int32_t k,
                                    pgx_tdma_plan** plan) {
  if (!a || !b || !c || !plan || n < 3 || n > PGX_LMAX - 8 || k != 2) return PGX_E_ARG;
  std::vector<double> tab;
  int rc = tdma_table(a, b, c, n, tab);
  if (rc) return rc;
  pgx_tdma_plan* p = new pgx_tdma_plan();
  p->n = n;
  rc = upload(tab, &p->tab);
  if (rc) {
    delete p;
    return rc;
  }
  *plan = p;
  return PGX_OK;
}

extern "C" int pgx_tdma_plan_destroy(pgx_tdma_plan* p) {
  if (!p) return PGX_E_PLAN;
  cudaFree(p->tab);
  delete p;
  return PGX_OK;
}

extern "C" int pgx_tdma_solve(const pgx_tdma_plan* p, const double* d, int64_t d_s0, int64_t d_s1, double* x,
                              int64_t x_s0, int64_t x_s1, int32_t nlines, int32_t axis, void* stream) {
  if (!p) return PGX_E_PLAN;
  if (!d || !x || nlines < 0 || axis < 0 || axis > 1) return PGX_E_ARG;
  pgx_program P;
  pgx_instance I;
  init_prog(P, I, axis);
  I.len[0] = nlines;
  I.len[1] = p->n;
  set_axis_arr(I, 0, d, d_s0, d_s1, axis, p->n, nlines);
  set_axis_arr(I, 1, x, x_s0, x_s1, axis, p->n, nlines);
  I.mat[0] = p->tab;
  P.nops = 3;
  P.ops[0] = mk(PGX_OP_LOAD, 0, -1, 0, -1, 1);
  P.ops[1] = mk(PGX_OP_TDMA2, 0, -1, -1, 0);
  P.ops[2] = mk(PGX_OP_STORE, 0, -1, 1);
  pick_tile(&P, nlines, p->n, 2, 0);
  return pgx_run(&P, &I, stream);
}

// ------------------------------------------------------------------ FDMA
struct pgx_fdma_plan {
  int n;
  double* tab;  // [l | dinv | u1 dinv | u2 dinv]
};

static void fdma_tab(const double* l, const double* d, const double* u1, const double* u2, int n,
                     std::vector<double>& tab, size_t off) {
  for (int i = 0; i < n; ++i) {
    tab[off + i] = (i >= 2 && l) ? l[i - 2] : 0.0;
    tab[off + n + i] = 1.0 / d[i];
    tab[off + 2 * n + i] = (i < n - 2 && u1) ? u1[i] / d[i] : 0.0;
    tab[off + 3 * n + i] = (i < n - 4 && u2) ? u2[i] / d[i] : 0.0;
  }
}

extern "C" int pgx_fdma_plan_create(const double* l, const double* d, const double* u1, const double* u2, int32_t n,
                                    pgx_fdma_plan** plan) {
  if (!d || !plan || n < 4 || n > PGX_LMAX - 8) return PGX_E_ARG;
  for (int i = 0; i < n; ++i)
    if (d[i] == 0.0) return PGX_E_SINGULAR;
  std::vector<double> tab(4 * (size_t)n, 0.0);
  fdma_tab(l, d, u1, u2, n, tab, 0);
  pgx_fdma_plan* p = new pgx_fdma_plan();
  p->n = n;
  int rc = upload(tab, &p->tab);
  if (rc) {
    delete p;
    return rc;
  }
  *plan = p;
  return PGX_OK;
}

extern "C" int pgx_twodma_plan_create(const double* d, const double* u, int32_t n, pgx_fdma_plan** plan) {
  return pgx_fdma_plan_create(nullptr, d, u, nullptr, n, plan);
}

extern "C" int pgx_fdma_plan_destroy(pgx_fdma_plan* p) {
  if (!p) return PGX_E_PLAN;
  cudaFree(p->tab);
  delete p;
  return PGX_OK;
}

static int fdma_solve_op(int code, const pgx_fdma_plan* p, double* x, int64_t s0, int64_t s1, int32_t nlines,
                         int32_t axis, void* stream);

extern "C" int pgx_fdma_solve(const pgx_fdma_plan* p, double* x, int64_t s0, int64_t s1, int32_t nlines, int32_t axis,
                              void* stream) {
  return fdma_solve_op(PGX_OP_FDMA, p, x, s0, s1, nlines, axis, stream);
}

extern "C" int pgx_fdma_solve_t(const pgx_fdma_plan* p, double* x, int64_t s0, int64_t s1, int32_t nlines,
                                int32_t axis, void* stream) {
  return fdma_solve_op(PGX_OP_FDMA_T, p, x, s0, s1, nlines, axis, stream);
}

static int fdma_solve_op(int code, const pgx_fdma_plan* p, double* x, int64_t s0, int64_t s1, int32_t nlines,
                         int32_t axis, void* stream) {
  if (!p) return PGX_E_PLAN;
  if (!x || nlines < 0 || axis < 0 || axis > 1) return PGX_E_ARG;
  pgx_program P;
  pgx_instance I;
  init_prog(P, I, axis);
  I.len[0] = nlines;
  I.len[1] = p->n;
  set_axis_arr(I, 0, x, s0, s1, axis, p->n, nlines);
  I.mat[0] = p->tab;
  P.nops = 3;
  P.ops[0] = mk(PGX_OP_LOAD, 0, -1, 0, -1, 1);
  P.ops[1] = mk(code, 0, -1, -1, 0);
  P.ops[2] = mk(PGX_OP_STORE, 0, -1, 0);
  pick_tile(&P, nlines, p->n, 2, 0);
  return pgx_run(&P, &I, stream);
}

// ---------------------------------------------------------------- Poisson
struct pgx_poisson_plan {
  int n, m;
  double* tab;  // m lines x [l | dinv | u1 dinv | u2 dinv] (n each)
};

// LU sweep of the four diagonals of an n x n band (init_fdma's recurrence).
static int band_lu(std::vector<double>& l, std::vector<double>& d, std::vector<double>& u1, std::vector<double>& u2,
                   int n) {
  for (int i = 2; i < n; ++i) {
    if (d[i - 2] == 0.0) return PGX_E_SINGULAR;
    l[i - 2] = l[i - 2] / d[i - 2];
    d[i] = d[i] - l[i - 2] * u1[i - 2];
    if (i < n - 2) u1[i] = u1[i] - l[i - 2] * u2[i - 2];
  }
  for (int i = 0; i < n; ++i)
    if (d[i] == 0.0) return PGX_E_SINGULAR;
  return PGX_OK;
}

extern "C" int pgx_poisson_plan_create(const double* A, const double* C, const double* lam, int32_t n, int32_t m,
                                       int32_t singular, pgx_poisson_plan** plan) {
  if (!A || !C || !lam || !plan || n < 5 || n > PGX_LMAX - 8 || m < 1) return PGX_E_ARG;
  std::vector<double> tab(4 * (size_t)n * m, 0.0);
  for (int j = 0; j < m; ++j) {
    const bool sing = singular && fabs(lam[j]) < 1e-10;
    const int o = sing ? 1 : 0;  // solve rows/cols o: of A + lam C
    const int ns = n - o;
    std::vector<double> l(ns, 0.0), d(ns, 0.0), u1(ns, 0.0), u2(ns, 0.0);
    auto el = [&](int r, int c) { return A[(size_t)(r + o) * n + c + o] + C[(size_t)(r + o) * n + c + o] * lam[j]; };
    for (int i = 0; i < ns; ++i) {
      d[i] = el(i, i);
      if (i >= 2) l[i - 2] = el(i, i - 2);
      if (i < ns - 2) u1[i] = el(i, i + 2);
      if (i < ns - 4) u2[i] = el(i, i + 4);
    }
    int rc = band_lu(l, d, u1, u2, ns);
    if (rc) return rc;
    const size_t base = (size_t)j * 4 * n;
    // place the ns-system at rows o..n-1 of a length-n table; row 0 of a singular
    // line has dinv = 0 so the sweep yields x_0 = 0 (fdma.f90:176-179)
    for (int i = 0; i < ns; ++i) {
      int g = i + o;
      tab[base + g] = i >= 2 ? l[i - 2] : 0.0;
      tab[base + n + g] = 1.0 / d[i];
      tab[base + 2 * n + g] = i < ns - 2 ? u1[i] / d[i] : 0.0;
      tab[base + 3 * n + g] = i < ns - 4 ? u2[i] / d[i] : 0.0;
    }
  }
  pgx_poisson_plan* p = new pgx_poisson_plan();
  p->n = n;
  p->m = m;
  int rc = upload(tab, &p->tab);
  if (rc) {
    delete p;
    return rc;
  }
  *plan = p;
  return PGX_OK;
}

extern "C" int pgx_poisson_plan_destroy(pgx_poisson_plan* p) {
  if (!p) return PGX_E_PLAN;
  cudaFree(p->tab);
  delete p;
  return PGX_OK;
}

static int poisson_solve_op(int code, const pgx_poisson_plan* p, double* x, int64_t s0, int64_t s1, int32_t axis,
                            void* stream);

extern "C" int pgx_poisson_solve(const pgx_poisson_plan* p, double* x, int64_t s0, int64_t s1, int32_t axis,
                                 void* stream) {
  return poisson_solve_op(PGX_OP_POISSON, p, x, s0, s1, axis, stream);
}

extern "C" int pgx_poisson_solve_t(const pgx_poisson_plan* p, double* x, int64_t s0, int64_t s1, int32_t axis,
                                   void* stream) {
  return poisson_solve_op(PGX_OP_POISSON_T, p, x, s0, s1, axis, stream);
}

static int poisson_solve_op(int code, const pgx_poisson_plan* p, double* x, int64_t s0, int64_t s1, int32_t axis,
                            void* stream) {
  if (!p) return PGX_E_PLAN;
  if (!x || axis < 0 || axis > 1) return PGX_E_ARG;
  pgx_program P;
  pgx_instance I;
  init_prog(P, I, axis);
  I.len[0] = p->m;
  I.len[1] = p->n;
  set_axis_arr(I, 0, x, s0, s1, axis, p->n, p->m);
  I.mat[0] = p->tab;
  P.nops = 3;
  P.ops[0] = mk(PGX_OP_LOAD, 0, -1, 0, -1, 1);
  P.ops[1] = mk(code, 0, -1, -1, 0);
  P.ops[2] = mk(PGX_OP_STORE, 0, -1, 0);
  pick_tile(&P, p->m, p->n, 2, 0);
  return pgx_run(&P, &I, stream);
}

// ----------------------------------------------------------------- matrices
struct pgx_matrix_plan {
  int rows, cols, banded, off0, ndiag;
  double* tab;
};

extern "C" int pgx_matrix_plan_create(const double* A, int32_t rows, int32_t cols, pgx_matrix_plan** plan) {
  if (!A || !plan || rows < 1 || cols < 1 || rows > PGX_LMAX - 8 || cols > PGX_LMAX - 8) return PGX_E_ARG;
  int lo = 1 << 30, hi = -(1 << 30), parity = -1;
  bool step2 = true;
  for (int r = 0; r < rows; ++r)
    for (int c = 0; c < cols; ++c)
      if (A[(size_t)r * cols + c] != 0.0) {
        int o = c - r;
        if (o < lo) lo = o;
        if (o > hi) hi = o;
        int par = ((o % 2) + 2) % 2;
        if (parity < 0) parity = par;
        else if (par != parity) step2 = false;
      }
  pgx_matrix_plan* p = new pgx_matrix_plan();
  p->rows = rows;
  p->cols = cols;
  std::vector<double> tab;
  if (lo > hi) {  // all zero: one zero diagonal
    lo = hi = 0;
  }
  int nd = (hi - lo) / 2 + 1;
  if (step2 && nd <= 8) {
    p->banded = 1;
    p->off0 = lo;
    p->ndiag = nd;
    tab.assign((size_t)nd * rows, 0.0);
    for (int d = 0; d < nd; ++d)
      for (int r = 0; r < rows; ++r) {
        int c = r + lo + 2 * d;
        if (c >= 0 && c < cols) tab[(size_t)d * rows + r] = A[(size_t)r * cols + c];
      }
  } else {
    p->banded = 0;
    p->off0 = 0;
    p->ndiag = 0;
    tab.assign(A, A + (size_t)rows * cols);
  }
  int rc = upload(tab, &p->tab);
  if (rc) {
    delete p;
    return rc;
  }
  *plan = p;
  return PGX_OK;
}

extern "C" int pgx_matrix_plan_destroy(pgx_matrix_plan* p) {
  if (!p) return PGX_E_PLAN;
  cudaFree(p->tab);
  delete p;
  return PGX_OK;
}

extern "C" int pgx_matrix_plan_is_banded(const pgx_matrix_plan* p) { return p ? p->banded : 0; }

extern "C" int pgx_matrix_apply(const pgx_matrix_plan* p, const double* in, int64_t in_s0, int64_t in_s1, double* out,
                                int64_t out_s0, int64_t out_s1, int32_t nlines, int32_t axis, void* stream) {
  if (!p) return PGX_E_PLAN;
  if (!in || !out || nlines < 0 || axis < 0 || axis > 1) return PGX_E_ARG;
  pgx_program P;
  pgx_instance I;
  init_prog(P, I, axis);
  I.len[0] = nlines;
  I.len[1] = p->cols;
  I.len[2] = p->rows;
  set_axis_arr(I, 0, in, in_s0, in_s1, axis, p->cols, nlines);
  set_axis_arr(I, 1, out, out_s0, out_s1, axis, p->rows, nlines);
  I.mat[0] = p->tab;
  P.nops = 3;
  P.ops[0] = mk(PGX_OP_LOAD, 0, -1, 0, -1, 1);
  if (p->banded) {
    P.ops[1] = mk(PGX_OP_BANDED, 0, p->off0, -1, 0, 2, p->ndiag);
  } else {
    P.ops[1] = mk(PGX_OP_DENSE, 0, -1, -1, 0, 2);
  }
  P.ops[2] = mk(PGX_OP_STORE, 0, -1, 1);
  pick_tile(&P, nlines, p->rows > p->cols ? p->rows : p->cols, 2, 0);
  return pgx_run(&P, &I, stream);
}
