// Line-program kernels for the pypde spectral-Galerkin time step on GB300 (sm_103a).
//
// One launch = one pass along one axis of a batch of 2-D arrays.  Every CTA owns
// a tile of `tb` lines of one instance.  The lines are loaded into shared
// memory "slots", a short program of 1-D operations (Chebyshev DCT-I via a
// mixed-radix FFT, Shen stencils, derivative recurrence, banded / dense
// operators, banded LU sweeps) runs on them, and results are stored back.
//
// All arithmetic is FP64.  On GB300 the FP64 pipe issues one warp instruction
// per ~64 cycles per SM sub-partition (1.26 TFLOP/s for the whole GPU) and a
// dependent DFMA has ~67 cycles of latency, so the kernels count FP64
// instructions, never divide in inner loops (reciprocals come from host-built
// tables), and keep index arithmetic in integer registers.
//
// Shared-memory invariant: every slot buffer holds zeros past the slot's
// logical length up to `lcap`, so ops may read a few elements past the end
// (banded sweeps read x[i+2], x[i+4]) without branches.

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <mutex>

#include "pgx.h"
#include "pgx_exact.cuh"

// Complex elements per line pair in each FFT buffer for DCT lengths up to n:
// n - 1 for the folded algorithm (even n - 1), 2(n - 1) for paired lines.
__host__ __device__ inline int pgx_fft_stride(int n) {
  if (n <= 1) return 0;
  return ((n - 1) & 1) == 0 ? (n - 1) : 2 * (n - 1);
}

__host__ __device__ inline bool pgx_has_dct(const pgx_program& P) {
  for (int o = 0; o < P.nops; ++o)
    if (P.ops[o].code == PGX_OP_DCT) return true;
  return false;
}

// Slots transformed together by one DCT op (op.b), the most of any DCT op of the program:
// the FFT buffers hold that many slots' line pairs.
__host__ __device__ inline int pgx_fft_slots(const pgx_program& P) {
  int fs = 1;
  for (int o = 0; o < P.nops; ++o)
    if (P.ops[o].code == PGX_OP_DCT && P.ops[o].b > fs) fs = P.ops[o].b;
  return fs;
}

// A program whose DCT ops each transform one slot, tiled in pairs of lines, with the folded transform
// (even n - 1: a pair's FFT data takes n - 1 complex values, at most its two lines of the slot) keeps
// its second FFT buffer in the spare slot: nothing lives there during a DCT op, and every op that
// later writes the spare overwrites or zeroes all of it.  One buffer less of shared memory per CTA.
__host__ __device__ inline bool pgx_fft_in_spare(const pgx_program& P) {
  if (P.fft_n <= 1 || pgx_fft_slots(P) != 1 || (P.tb & 1)) return false;
  return 2LL * pgx_fft_stride(P.fft_n) * ((P.tb + 1) / 2) <= (long long)P.tb * P.lcap;
}

// Every DCT op of the program runs in its slot's own lines and the spare (PGX_DCT_SLOT): no FFT buffers.
__host__ __device__ inline bool pgx_fft_in_slot(const pgx_program& P) {
  bool any = false;
  for (int o = 0; o < P.nops; ++o)
    if (P.ops[o].code == PGX_OP_DCT) {
      if (!(P.ops[o].k & PGX_DCT_SLOT)) return false;
      any = true;
    }
  return any && !(P.tb & 1);
}

namespace pgx {

// 2k for k < PGX_LMAX: multipliers of the derivative recurrence, read through
// the constant cache (lanes of a warp read the same k in lockstep).
struct TwoK {
  double v[PGX_LMAX];
};
constexpr TwoK make_twok() {
  TwoK t{};
  for (int i = 0; i < PGX_LMAX; ++i) t.v[i] = 2.0 * i;
  return t;
}
__constant__ TwoK c_twok = make_twok();

struct Ctx {
  double* sm;       // slot buffers
  double2* f0;      // FFT ping buffer
  double2* f1;      // FFT pong buffer
  double* ybuf;     // one scalar per line (DCT-I: y_1 of the folded algorithm)
  int tb, lcap, nthreads, tid;
  int fft_stride;   // complex elements per pair in the FFT buffers
  int l0, nlines;   // first line of the tile, lines of the instance
  int phys[PGX_MAX_SLOTS + 1];
  int slen[PGX_MAX_SLOTS];
  int spare;
};

__device__ __forceinline__ double* slot_ptr(const Ctx& c, int s) {
  return c.sm + (size_t)c.phys[s] * c.tb * c.lcap;
}
// Slot s0 + sl of a multi-slot op whose slot s0 is x0: sl == 0 (every one-slot op) reads no slot map.
__device__ __forceinline__ double* op_slot(const Ctx& c, double* x0, int s0, int sl) {
  return sl == 0 ? x0 : slot_ptr(c, s0 + sl);
}
__device__ __forceinline__ double* spare_ptr(const Ctx& c) {
  return c.sm + (size_t)c.spare * c.tb * c.lcap;
}
__device__ __forceinline__ void swap_spare(Ctx& c, int s) {
  int t = c.phys[s];
  c.phys[s] = c.spare;
  c.spare = t;
}

__device__ __forceinline__ double op_alpha(const pgx_op& op, const pgx_instance& I) {
  return op.par >= 0 ? op.alpha * I.par[op.par] : op.alpha;
}

// Geometry of array `a` seen from a pass along `axis`.
struct View {
  double* p;
  int64_t se, sl;  // element stride, line stride
  int ne, nl;      // elements per line, lines
};
__device__ __forceinline__ View view_of(const pgx_array& a, int axis) {
  View v;
  v.p = a.ptr;
  if (axis == 0) {
    v.se = a.s0; v.sl = a.s1; v.ne = a.n0; v.nl = a.n1;
  } else {
    v.se = a.s1; v.sl = a.s0; v.ne = a.n1; v.nl = a.n0;
  }
  return v;
}

// Zero [from, lcap) of every line of buffer `b`.
__device__ void zero_tail(const Ctx& c, double* b, int from) {
  const int c_tb = c.tb;
  const int c_lcap = c.lcap;
  const int c_nthreads = c.nthreads;
  const int c_tid = c.tid;
  int w = c_lcap - from;
  if (w <= 0) return;
  for (int idx = c_tid; idx < c_tb * w; idx += c_nthreads) {
    int t = idx / w, i = from + idx % w;
    b[t * c_lcap + i] = 0.0;
  }
}

// ------------------------------------------------------------------ load/store
// mode 0: slot = alpha*arr (length n, zero beyond the array), 1: +=, 2: *=
template <int KU>
__device__ void op_load(Ctx& c, const pgx_op& op, const pgx_instance& I, int axis, int mode) {
  const int c_tb = c.tb;
  const int c_lcap = c.lcap;
  const int c_nthreads = c.nthreads;
  const int c_tid = c.tid;
  const int c_l0 = c.l0;
  const int c_nlines = c.nlines;
  const View v = view_of(I.arr[op.arr], axis);
  const double alpha = op_alpha(op, I);
  int n;
  if (mode == 0) {
    n = I.len[op.len];
    c.slen[op.a] = n;
  } else {
    n = c.slen[op.a];
  }
  double* s = slot_ptr(c, op.a);
  const int tb = c_tb;
  const bool contig = (v.se == 1);
  const int total = tb * n;
  // up to kU elements a thread per round, all their global loads issued before the first store to
  // the slot: the stores go through generic pointers, which the compiler may not move loads across,
  // so one element at a time would wait out a full memory latency per element (the build for
  // launches of fewer CTAs than SMs, KU = 1, keeps the shorter single-element loop)
  constexpr int kU = KU;
  if (total <= c_nthreads) {  // at most one element a thread (single instances, short lines)
    if (c_tid < total) {
      int t, i;
      if (contig) { t = c_tid / n; i = c_tid - t * n; }
      else { i = c_tid / tb; t = c_tid - i * tb; }
      const int line = c_l0 + t;
      double x = 0.0;
      if (i < v.ne && line < v.nl && line < c_nlines) x = v.p[(int64_t)i * v.se + (int64_t)line * v.sl];
      double* d = s + t * c_lcap + i;
      if (mode == 0) *d = alpha == 1.0 ? x : alpha * x;
      else if (mode == 1) *d = fma(alpha, x, *d);
      else *d = (alpha == 1.0 ? x : alpha * x) * (*d);
    }
    if (mode == 0) zero_tail(c, s, n);
    return;
  }
  for (int base = c_tid; base < total; base += kU * c_nthreads) {
    double x[kU];
    int off[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int idx = base + u * c_nthreads;
      x[u] = 0.0;
      off[u] = -1;
      if (idx < total) {
        int t, i;
        if (contig) { t = idx / n; i = idx - t * n; }
        else { i = idx / tb; t = idx - i * tb; }
        const int line = c_l0 + t;
        off[u] = t * c_lcap + i;
        if (i < v.ne && line < v.nl && line < c_nlines) x[u] = v.p[(int64_t)i * v.se + (int64_t)line * v.sl];
      }
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      if (off[u] < 0) continue;
      double* d = s + off[u];
      if (mode == 0) *d = alpha == 1.0 ? x[u] : alpha * x[u];
      else if (mode == 1) *d = fma(alpha, x[u], *d);
      else *d = (alpha == 1.0 ? x[u] : alpha * x[u]) * (*d);
    }
  }
  if (mode == 0) zero_tail(c, s, n);  // [n, lcap) of every line: no element the loop writes
}

template <int KU>
__device__ void op_store(const Ctx& c, const pgx_op& op, const pgx_instance& I, int axis, bool add) {
  const int c_tb = c.tb;
  const int c_lcap = c.lcap;
  const int c_nthreads = c.nthreads;
  const int c_tid = c.tid;
  const int c_l0 = c.l0;
  const int c_nlines = c.nlines;
  const View v = view_of(I.arr[op.arr], axis);
  const double alpha = op_alpha(op, I);
  const double* s = slot_ptr(c, op.a);
  const int n = v.ne;
  const int tb = c_tb;
  const bool contig = (v.se == 1);
  const int total = tb * n;
  // up to kU elements a thread per round, every load (the slot's and, to accumulate, the array's)
  // before the first store: one memory latency per round, not per element
  constexpr int kU = KU;
  if (total <= c_nthreads) {  // at most one element a thread (single instances, short lines)
    if (c_tid < total) {
      int t, i;
      if (contig) { t = c_tid / n; i = c_tid - t * n; }
      else { i = c_tid / tb; t = c_tid - i * tb; }
      const int line = c_l0 + t;
      if (line < v.nl && line < c_nlines) {
        const double x = s[t * c_lcap + i];
        double* d = v.p + (int64_t)i * v.se + (int64_t)line * v.sl;
        if (add) *d = fma(alpha, x, *d);
        else *d = alpha == 1.0 ? x : alpha * x;
      }
    }
    return;
  }
  for (int base = c_tid; base < total; base += kU * c_nthreads) {
    double x[kU], old[kU];
    double* dp[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int idx = base + u * c_nthreads;
      dp[u] = nullptr;
      x[u] = old[u] = 0.0;
      if (idx < total) {
        int t, i;
        if (contig) { t = idx / n; i = idx - t * n; }
        else { i = idx / tb; t = idx - i * tb; }
        const int line = c_l0 + t;
        if (line < v.nl && line < c_nlines) {
          x[u] = s[t * c_lcap + i];
          dp[u] = v.p + (int64_t)i * v.se + (int64_t)line * v.sl;
          if (add) old[u] = *dp[u];
        }
      }
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      if (!dp[u]) continue;
      if (add) *dp[u] = fma(alpha, x[u], old[u]);
      else *dp[u] = alpha == 1.0 ? x[u] : alpha * x[u];
    }
  }
}

// ------------------------------------------------------------- pointwise ops
__device__ void op_pointwise(Ctx& c, const pgx_op& op, const pgx_instance& I) {
  const int c_tb = c.tb;
  const int c_lcap = c.lcap;
  const int c_nthreads = c.nthreads;
  const int c_tid = c.tid;
  const double alpha = op_alpha(op, I);
  double* a = slot_ptr(c, op.a);
  const double* b = op.b >= 0 ? slot_ptr(c, op.b) : nullptr;
  int n = c.slen[op.a];
  if (op.code != PGX_OP_SCALE) {
    int nb = c.slen[op.b];
    if (op.code == PGX_OP_COPY) n = nb;
    else if (nb > n) n = nb;
    c.slen[op.a] = n;
  }
  for (int idx = c_tid; idx < c_tb * n; idx += c_nthreads) {
    int t = idx / n, i = idx - t * n;
    int o = t * c_lcap + i;
    switch (op.code) {
      case PGX_OP_SCALE: a[o] *= alpha; break;
      case PGX_OP_AXPY: a[o] = fma(alpha, b[o], a[o]); break;
      case PGX_OP_MUL: a[o] = (alpha == 1.0 ? b[o] : alpha * b[o]) * a[o]; break;
      case PGX_OP_COPY: a[o] = alpha == 1.0 ? b[o] : alpha * b[o]; break;
    }
  }
  if (op.code == PGX_OP_COPY) zero_tail(c, a, n);  // [n, lcap): no element the loop reads or writes
}

__device__ void op_setlen(Ctx& c, const pgx_op& op, const pgx_instance& I) {
  int n = I.len[op.len];
  int old = c.slen[op.a];
  if (n < old) zero_tail(c, slot_ptr(c, op.a), n);
  c.slen[op.a] = n;
}

// ------------------------------------------------------------------ stencils
// u_i = v_i [i < M] + s_{i-2} v_{i-2} [i >= 2],  s = S[i+2, i] sub-diagonal table.
template <int KU>
__device__ void op_stencil(Ctx& c, const pgx_op& op, const pgx_instance& I) {
  const int c_tb = c.tb;
  const int c_lcap = c.lcap;
  const int c_nthreads = c.nthreads;
  const int c_tid = c.tid;
  const double* sd = I.mat[op.mat];
  const double* x = slot_ptr(c, op.a);
  double* y = spare_ptr(c);
  const int M = c.slen[op.a], N = M + 2;
  const int total = c_tb * c_lcap;
  constexpr int kU = KU;  // the table loads of kU elements before their stores
  for (int base = c_tid; base < total; base += kU * c_nthreads) {
    double r[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int idx = base + u * c_nthreads;
      r[u] = 0.0;
      if (idx < total) {
        const int t = idx / c_lcap, i = idx - t * c_lcap;
        if (i < N) {
          const double* xl = x + t * c_lcap;
          r[u] = i < M ? xl[i] : 0.0;
          if (i >= 2) r[u] = fma(__ldg(sd + i - 2), xl[i - 2], r[u]);
        }
      }
    }
#pragma unroll
    for (int u = 0; u < kU; ++u)
      if (base + u * c_nthreads < total) y[base + u * c_nthreads] = r[u];
  }
  swap_spare(c, op.a);
  c.slen[op.a] = N;
}

// (S^T u)_i = u_i + s_i u_{i+2},  i < N-2.
template <int KU>
__device__ void op_stencil_t(Ctx& c, const pgx_op& op, const pgx_instance& I) {
  const int c_tb = c.tb;
  const int c_lcap = c.lcap;
  const int c_nthreads = c.nthreads;
  const int c_tid = c.tid;
  const double* sd = I.mat[op.mat];
  const double* x = slot_ptr(c, op.a);
  double* y = spare_ptr(c);
  const int N = c.slen[op.a], M = N - 2;
  const int total = c_tb * c_lcap;
  constexpr int kU = KU;  // the table loads of kU elements before their stores
  for (int base = c_tid; base < total; base += kU * c_nthreads) {
    double r[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int idx = base + u * c_nthreads;
      r[u] = 0.0;
      if (idx < total) {
        const int t = idx / c_lcap, i = idx - t * c_lcap;
        if (i < M) {
          const double* xl = x + t * c_lcap;
          r[u] = fma(__ldg(sd + i), xl[i + 2], xl[i]);
        }
      }
    }
#pragma unroll
    for (int u = 0; u < kU; ++u)
      if (base + u * c_nthreads < total) y[base + u * c_nthreads] = r[u];
  }
  swap_spare(c, op.a);
  c.slen[op.a] = M;
}

// ------------------------------------------------ sequential parity chains
// A chain op sweeps `ns` consecutive slots a, a+1, ... at once (independent
// solves of one pass run concurrently, so every warp has chains to run).
// Thread (s, p, t) owns the chain of line t of slot a+s with indices = p (mod 2).
__device__ __forceinline__ bool chain_of(const Ctx& c, int ns, int& s, int& t, int& p) {
  if (c.tid >= 2 * c.tb * ns) return false;
  s = c.tid / (2 * c.tb);
  int r = c.tid - s * 2 * c.tb;
  p = r / c.tb;
  t = r - p * c.tb;
  return true;
}
__device__ __forceinline__ int nslot_of(const pgx_op& op) { return op.b > 1 ? op.b : 1; }

// ------------------------------------------------- warp-parallel recurrences
// With few lines (one large instance) a chain per thread leaves the GPU idle while
// each chain walks n/2 dependent steps.  In the warp mode of a chain op
// (op.k & PGX_CHAIN_WARP) one warp solves one (line, parity) chain: the lanes own
// consecutive segments, each lane composes its segment's affine map, the maps are
// scanned across the warp with shuffles, and every lane re-runs its segment from
// its exact incoming state.  The work grows ~3x, the dependent path shrinks from
// n/2 steps to ~n/32 + 5 combine levels.
constexpr unsigned FULLMASK = 0xffffffffu;

// y_q = b(q) + a(q) y_{q-1} for q = 0..m-1 (recurrence order), y_{-1} = 0; put(q, y).
template <class FA, class FB, class FP>
__device__ __forceinline__ void warp_rec1(int m, int lane, FA a, FB b, FP put) {
  const int C = (m + 31) >> 5;
  const int q0 = min(lane * C, m), q1 = min(q0 + C, m);
  double A = 1.0, B = 0.0;
  for (int q = q0; q < q1; ++q) {
    const double aq = a(q);
    B = fma(aq, B, b(q));
    A *= aq;
  }
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double Ap = __shfl_up_sync(FULLMASK, A, o), Bp = __shfl_up_sync(FULLMASK, B, o);
    if (lane >= o) {
      B = fma(A, Bp, B);
      A *= Ap;
    }
  }
  double y = __shfl_up_sync(FULLMASK, B, 1);
  if (lane == 0) y = 0.0;
  for (int q = q0; q < q1; ++q) {
    y = fma(a(q), y, b(q));
    put(q, y);
  }
}

// y_q = b(q) + a1(q) y_{q-1} + a2(q) y_{q-2}, y_{-1} = y_{-2} = 0; put(q, y).
// Segment maps act on the state (y_q, y_{q-1}): s_out = M s_in + c.
template <class FA1, class FA2, class FB, class FP>
__device__ __forceinline__ void warp_rec2(int m, int lane, FA1 a1, FA2 a2, FB b, FP put) {
  const int C = (m + 31) >> 5;
  const int q0 = min(lane * C, m), q1 = min(q0 + C, m);
  double m00 = 1.0, m01 = 0.0, m10 = 0.0, m11 = 1.0, c0 = 0.0, c1 = 0.0;
  for (int q = q0; q < q1; ++q) {
    const double x1 = a1(q), x2 = a2(q);
    const double n00 = fma(x2, m10, x1 * m00), n01 = fma(x2, m11, x1 * m01);
    const double nc0 = fma(x2, c1, fma(x1, c0, b(q)));
    m10 = m00;
    m11 = m01;
    c1 = c0;
    m00 = n00;
    m01 = n01;
    c0 = nc0;
  }
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double p00 = __shfl_up_sync(FULLMASK, m00, o), p01 = __shfl_up_sync(FULLMASK, m01, o);
    const double p10 = __shfl_up_sync(FULLMASK, m10, o), p11 = __shfl_up_sync(FULLMASK, m11, o);
    const double pc0 = __shfl_up_sync(FULLMASK, c0, o), pc1 = __shfl_up_sync(FULLMASK, c1, o);
    if (lane >= o) {  // (M, c) after (P, pc): (M P, M pc + c)
      const double r00 = fma(m01, p10, m00 * p00), r01 = fma(m01, p11, m00 * p01);
      const double r10 = fma(m11, p10, m10 * p00), r11 = fma(m11, p11, m10 * p01);
      const double s0 = fma(m01, pc1, fma(m00, pc0, c0)), s1 = fma(m11, pc1, fma(m10, pc0, c1));
      m00 = r00;
      m01 = r01;
      m10 = r10;
      m11 = r11;
      c0 = s0;
      c1 = s1;
    }
  }
  double y1 = __shfl_up_sync(FULLMASK, c0, 1), y2 = __shfl_up_sync(FULLMASK, c1, 1);
  if (lane == 0) y1 = y2 = 0.0;
  for (int q = q0; q < q1; ++q) {
    const double y = fma(a2(q), y2, fma(a1(q), y1, b(q)));
    y2 = y1;
    y1 = y;
    put(q, y);
  }
}

// The chain of parity p of an n-point line, x[p + 2k], k < m = (n - p + 1) / 2.
__device__ __forceinline__ void fdma_chain_warp(double* x, const double* tab, int n, int p, int lane) {
  const double* l = tab;
  const double* dinv = tab + n;
  const double* u1 = tab + 2 * n;
  const double* u2 = tab + 3 * n;
  const int m = (n - p + 1) >> 1;
  // L: y_k = x_k - l_k y_{k-1}
  warp_rec1(m, lane, [&](int q) { return -__ldg(l + p + 2 * q); }, [&](int q) { return x[p + 2 * q]; },
            [&](int q, double y) { x[p + 2 * q] = y; });
  __syncwarp();
  // U (from the top): v_i = x_i dinv_i - (u1 dinv)_i v_{i+2} - (u2 dinv)_i v_{i+4}
  warp_rec2(m, lane, [&](int q) { return -__ldg(u1 + p + 2 * (m - 1 - q)); },
            [&](int q) { return -__ldg(u2 + p + 2 * (m - 1 - q)); },
            [&](int q) { const int i = p + 2 * (m - 1 - q); return x[i] * __ldg(dinv + i); },
            [&](int q, double y) { x[p + 2 * (m - 1 - q)] = y; });
}

__device__ __forceinline__ void fdma_t_chain_warp(double* x, const double* tab, int n, int p, int lane) {
  const double* l = tab;
  const double* dinv = tab + n;
  const double* u1 = tab + 2 * n;
  const double* u2 = tab + 3 * n;
  const int m = (n - p + 1) >> 1;
  // U^T on zeta = z / dinv: zeta_i = x_i - (u1 dinv)_{i-2} zeta_{i-2} - (u2 dinv)_{i-4} zeta_{i-4}; z = zeta dinv
  warp_rec2(m, lane, [&](int q) { const int i = p + 2 * q; return i >= 2 ? -__ldg(u1 + i - 2) : 0.0; },
            [&](int q) { const int i = p + 2 * q; return i >= 4 ? -__ldg(u2 + i - 4) : 0.0; },
            [&](int q) { return x[p + 2 * q]; },
            [&](int q, double y) { const int i = p + 2 * q; x[i] = y * __ldg(dinv + i); });
  __syncwarp();
  // L^T (from the top): x_i = z_i - l_{i+2} x_{i+2}
  warp_rec1(m, lane, [&](int q) { const int i = p + 2 * (m - 1 - q); return i + 2 < n ? -__ldg(l + i + 2) : 0.0; },
            [&](int q) { return x[p + 2 * (m - 1 - q)]; }, [&](int q, double y) { x[p + 2 * (m - 1 - q)] = y; });
}

__device__ __forceinline__ void tdma_chain_warp(double* x, const double* tab, int n, int p, int lane) {
  const int m = (n - p + 1) >> 1;
  // g_i = r_i x_i - (a r)_i g_{i-2};  x_i = g_i - w_i x_{i+2}
  warp_rec1(m, lane, [&](int q) { return -__ldg(tab + 3 * (p + 2 * q)); },
            [&](int q) { const int i = p + 2 * q; return x[i] * __ldg(tab + 3 * i + 1); },
            [&](int q, double y) { x[p + 2 * q] = y; });
  __syncwarp();
  warp_rec1(m, lane, [&](int q) { return -__ldg(tab + 3 * (p + 2 * (m - 1 - q)) + 2); },
            [&](int q) { return x[p + 2 * (m - 1 - q)]; }, [&](int q, double y) { x[p + 2 * (m - 1 - q)] = y; });
}

// (S^T S) x = d with the offset-2 TDMA; table interleaved per index i as
// (aa_i, rden_i, w_i), so one long table serves every system length n:
//   g_i = (d_i - aa_i g_{i-2}) rden_i,  x_j = g_j - w_j x_{j+2}.
// The last two w_i of a chain multiply x_{n}, x_{n+1} = 0 and are never used.
__device__ void op_tdma2(Ctx& c, const pgx_op& op, const pgx_instance& I) {
  const int c_tb = c.tb;
  const int c_lcap = c.lcap;
  const int c_nthreads = c.nthreads;
  const int c_tid = c.tid;
  int s, t, p;
  const int ns = nslot_of(op);
  if (op.k & PGX_CHAIN_WARP) {
    const int lane = c_tid & 31, nw = c_nthreads >> 5;
    for (int w = c_tid >> 5; w < 2 * c_tb * ns; w += nw) {
      s = w / (2 * c_tb);
      const int r = w - s * 2 * c_tb;
      p = r / c_tb;
      t = r - p * c_tb;
      const int n = c.slen[op.a + s];
      if (p >= n) continue;
      tdma_chain_warp(slot_ptr(c, op.a + s) + t * c_lcap, I.mat[op.mat], n, p, lane);
    }
    return;
  }
  for (int base = 0; base < 2 * c_tb * ns; base += c_nthreads) {
    Ctx cc = c;
    cc.tid = c_tid + base;
    if (!chain_of(cc, ns, s, t, p)) continue;
    const int n = c.slen[op.a + s];
    if (p >= n) continue;
    const double* tab = I.mat[op.mat];
    double* x = slot_ptr(c, op.a + s) + t * c_lcap;
    double g = 0.0;
    int i = p;
    for (; i < n; i += 2) {  // g_i = r_i x_i - (a r)_i g_{i-2}: one dependent FMA per step
      g = fma(-__ldg(tab + 3 * i), g, x[i] * __ldg(tab + 3 * i + 1));
      x[i] = g;
    }
    double xn = 0.0;
    for (i -= 2; i >= 0; i -= 2) {
      xn = fma(-__ldg(tab + 3 * i + 2), xn, x[i]);
      x[i] = xn;
    }
  }
}

// Chebyshev derivative in place (differentiate_cheby.f90:28-53):
//   dc_{n-1} = 0, dc_j = dc_{j+2} + 2(j+1) c_{j+1} (j = n-2..1), dc_0 = dc_2/2 + c_1,
// i.e. dc_j = S_{(j+1) mod 2}(j+1) with S_p(i) = sum_{k >= i, k = p mod 2} 2k c_k.
// One warp per (slot, line): each lane owns a contiguous chunk, the chunk totals of
// both parity classes are suffix-scanned across the warp, then every lane walks its
// chunk backwards.  Depth ~ n/32 + 5 dependent adds instead of n.
// lanes per line for per-line phases of a warp that owns nl lines (2 <= L <= 32): the warp's
// 32 lanes cover all its lines at once
__device__ __forceinline__ int lanes_per_line(int nl) {
  int L = 32;
  while (L > 2 && L * nl > 32) L >>= 1;
  return L;
}

// Lines of a per-line op over ns slots: warp w takes lines [w per, (w + 1) per), then every
// nw * per further; L lanes a line (the lanes of one line form an aligned group of L).
struct LineLanes {
  int L, per, grp, sub, first, stride, nl;
};
__device__ __forceinline__ LineLanes line_lanes(const Ctx& c, int nl) {
  LineLanes g;
  const int nw = c.nthreads >> 5, lane = c.tid & 31;
  g.L = lanes_per_line((nl + nw - 1) / nw);
  g.per = 32 / g.L;
  g.grp = lane / g.L;
  g.sub = lane & (g.L - 1);
  g.first = (c.tid >> 5) * g.per;
  g.stride = nw * g.per;
  g.nl = nl;
  return g;
}

__device__ void op_diff(Ctx& c, const pgx_op& op) {
  const int c_tb = c.tb;
  const int c_lcap = c.lcap;
  const int ns = nslot_of(op);
  const LineLanes g = line_lanes(c, ns * c_tb);
  for (int base = g.first; base < g.nl; base += g.stride) {  // the same trip count for the whole warp
    const int w = base + g.grp;
    const bool valid = w < g.nl;
    const int s = valid ? w / c_tb : 0, t = valid ? w - s * c_tb : 0;
    const int n = valid ? c.slen[op.a + s] : 0;
    double* x = slot_ptr(c, op.a + s) + t * c_lcap;
    const int chunk = (n + g.L - 1) / g.L;
    const int a = min(g.sub * chunk, n), b = min(a + chunk, n);
    for (int rep = 0; rep < op.k; ++rep) {
      double tot[2] = {0.0, 0.0};
      for (int i = a; i < b; ++i) tot[i & 1] = fma(c_twok.v[i], x[i], tot[i & 1]);
      const double c1 = valid ? x[1] : 0.0;
      // exclusive suffix sums of the chunk totals over the lanes above this one (of this line)
      double in0 = tot[0], in1 = tot[1];
      for (int o = 1; o < g.L; o <<= 1) {
        const double v0 = __shfl_down_sync(0xffffffffu, in0, o, g.L);
        const double v1 = __shfl_down_sync(0xffffffffu, in1, o, g.L);
        if (g.sub + o < g.L) {
          in0 += v0;
          in1 += v1;
        }
      }
      double acc[2] = {in0 - tot[0], in1 - tot[1]};  // S_p(b)
      __syncwarp();
      for (int i = b - 1; i >= a; --i) {
        const double wi = c_twok.v[i] * x[i];
        x[i] = acc[(i + 1) & 1];  // dc_i = S_{(i+1) mod 2}(i+1)
        acc[i & 1] += wi;
      }
      __syncwarp();
      if (valid && g.sub == 0) x[0] = fma(0.5, n > 2 ? x[2] : 0.0, c1);
      __syncwarp();
    }
  }
}

// Transpose of the derivative recurrence (adjoint of op_diff), in place:
//   (D^T y)_i = 2i sum_{1 <= j < i, j = i+1 mod 2} y_j + y_0 [i odd] (1 if i = 1 else i).
// Forward prefix sums per parity class, L lanes a line.
__device__ void op_diff_t(Ctx& c, const pgx_op& op) {
  const int c_tb = c.tb;
  const int c_lcap = c.lcap;
  const int ns = nslot_of(op);
  const LineLanes g = line_lanes(c, ns * c_tb);
  for (int base = g.first; base < g.nl; base += g.stride) {
    const int w = base + g.grp;
    const bool valid = w < g.nl;
    const int s = valid ? w / c_tb : 0, t = valid ? w - s * c_tb : 0;
    const int n = valid ? c.slen[op.a + s] : 0;
    double* x = slot_ptr(c, op.a + s) + t * c_lcap;
    const int chunk = (n + g.L - 1) / g.L;
    const int a = min(g.sub * chunk, n), b = min(a + chunk, n);
    for (int rep = 0; rep < op.k; ++rep) {
      double tot[2] = {0.0, 0.0};
      for (int i = max(a, 1); i < b; ++i) tot[i & 1] += x[i];
      const double y0 = valid ? x[0] : 0.0;
      double in0 = tot[0], in1 = tot[1];
      for (int o = 1; o < g.L; o <<= 1) {
        const double v0 = __shfl_up_sync(0xffffffffu, in0, o, g.L);
        const double v1 = __shfl_up_sync(0xffffffffu, in1, o, g.L);
        if (g.sub >= o) {
          in0 += v0;
          in1 += v1;
        }
      }
      double acc[2] = {in0 - tot[0], in1 - tot[1]};  // sums over j < a, j >= 1
      __syncwarp();
      for (int i = a; i < b; ++i) {
        const double yi = x[i];
        double v = c_twok.v[i] * acc[(i + 1) & 1];
        if (i & 1) v = fma(i == 1 ? 1.0 : 0.5 * c_twok.v[i], y0, v);
        x[i] = v;
        if (i >= 1) acc[i & 1] += yi;
      }
      __syncwarp();
    }
  }
}

// In-place banded LU sweep for offsets -2, 0, +2, +4 (fdma.f90:1-38) with
// factors [l | dinv | u1 | u2] (each n, zero-padded, l[i] couples x_i to x_{i-2}):
//   forward  x_i -= l_i x_{i-2};   backward x_i = (x_i - u1_i x_{i+2} - u2_i x_{i+4}) dinv_i
// A chain step waits for its factor loads; the per-line Poisson factors are touched once,
// so they would come from L2 at every step.  Each step therefore asks L1 for the factors
// PF elements ahead (in-bounds addresses only; a prefetch is a hint and changes no result).
constexpr int PF = 32;
__device__ __forceinline__ void prefetch_l1(const double* a) { asm volatile("prefetch.L1 [%0];" ::"l"(a)); }

__device__ __forceinline__ void fdma_chain(double* x, const double* tab, int n, int p) {
  const double* l = tab;
  const double* dinv = tab + n;
  const double* u1 = tab + 2 * n;
  const double* u2 = tab + 3 * n;
  double prev = x[p];
  int i = p + 2;
  for (; i < n; i += 2) {
    if (i + PF < n) prefetch_l1(l + i + PF);
    prev = fma(-__ldg(l + i), prev, x[i]);
    x[i] = prev;
  }
  double x2 = 0.0, x4 = 0.0;
  for (i -= 2; i >= 0; i -= 2) {  // u1, u2 hold u dinv: one FMA on the x2 dependency
    if (i >= PF) {
      prefetch_l1(dinv + i - PF);
      prefetch_l1(u1 + i - PF);
      prefetch_l1(u2 + i - PF);
    }
    const double w = fma(-__ldg(u2 + i), x4, x[i] * __ldg(dinv + i));
    const double v = fma(-__ldg(u1 + i), x2, w);
    x[i] = v;
    x4 = x2;
    x2 = v;
  }
}

// FDMA over ns slots: slot a+s uses factor table mat+s.  POISSON (per_line):
// single table with per-line factors.
// Transposed solve A^T x = b with the factors of A = L U (adjoint of fdma_chain):
//   U^T z = b (forward):  z_i = (b_i - u1_{i-2} z_{i-2} - u2_{i-4} z_{i-4}) dinv_i, run on
//                         zeta_i = z_i / dinv_i = b_i - (u1 dinv)_{i-2} zeta_{i-2} - (u2 dinv)_{i-4} zeta_{i-4}
//   L^T x = z (backward): x_i = z_i - l_{i+2} x_{i+2}
__device__ __forceinline__ void fdma_t_chain(double* x, const double* tab, int n, int p) {
  const double* l = tab;
  const double* dinv = tab + n;
  const double* u1 = tab + 2 * n;  // u1 dinv
  const double* u2 = tab + 3 * n;  // u2 dinv
  double z2 = 0.0, z4 = 0.0;       // zeta_{i-2}, zeta_{i-4}
  int i = p;
  for (; i < n; i += 2) {
    if (i + PF < n) {
      prefetch_l1(dinv + i + PF);
      prefetch_l1(u1 + i + PF - 2);
      prefetch_l1(u2 + i + PF - 4);
    }
    double v = x[i];
    if (i >= 4) v = fma(-__ldg(u2 + i - 4), z4, v);
    if (i >= 2) v = fma(-__ldg(u1 + i - 2), z2, v);
    x[i] = v * __ldg(dinv + i);
    z4 = z2;
    z2 = v;
  }
  double xn = 0.0;
  for (i -= 2; i >= 0; i -= 2) {
    if (i >= PF) prefetch_l1(l + i + 2 - PF);
    const double li = (i + 2 < n) ? __ldg(l + i + 2) : 0.0;
    xn = fma(-li, xn, x[i]);
    x[i] = xn;
  }
}

__device__ void op_fdma(Ctx& c, const pgx_op& op, const pgx_instance& I, bool per_line, bool transpose = false) {
  const int c_tb = c.tb;
  const int c_lcap = c.lcap;
  const int c_nthreads = c.nthreads;
  const int c_tid = c.tid;
  const int c_l0 = c.l0;
  const int c_nlines = c.nlines;
  int s, t, p;
  const int ns = nslot_of(op);
  if (op.k & PGX_CHAIN_WARP) {
    const int lane = c_tid & 31, nw = c_nthreads >> 5;
    for (int w = c_tid >> 5; w < 2 * c_tb * ns; w += nw) {
      s = w / (2 * c_tb);
      const int r = w - s * 2 * c_tb;
      p = r / c_tb;
      t = r - p * c_tb;
      const int n = c.slen[op.a + s];
      const int line = c_l0 + t;
      if (p >= n || line >= c_nlines) continue;
      const double* tab = I.mat[op.mat + (per_line ? 0 : s)];
      if (per_line) tab += (size_t)line * 4 * n;
      double* x = slot_ptr(c, op.a + s) + t * c_lcap;
      if (transpose) fdma_t_chain_warp(x, tab, n, p, lane);
      else fdma_chain_warp(x, tab, n, p, lane);
    }
    return;
  }
  for (int base = 0; base < 2 * c_tb * ns; base += c_nthreads) {
    Ctx cc = c;
    cc.tid = c_tid + base;
    if (!chain_of(cc, ns, s, t, p)) continue;
    const int n = c.slen[op.a + s];
    const int line = c_l0 + t;
    if (p >= n || line >= c_nlines) continue;
    const double* tab = I.mat[op.mat + (per_line ? 0 : s)];
    if (per_line) tab += (size_t)line * 4 * n;
    if (transpose) fdma_t_chain(slot_ptr(c, op.a + s) + t * c_lcap, tab, n, p);
    else fdma_chain(slot_ptr(c, op.a + s) + t * c_lcap, tab, n, p);
  }
}

// --------------------------------------------------------- banded / dense
template <int KU>
__device__ void op_banded(Ctx& c, const pgx_op& op, const pgx_instance& I) {
  const int c_tb = c.tb;
  const int c_lcap = c.lcap;
  const int c_nthreads = c.nthreads;
  const int c_tid = c.tid;
  const double* A = I.mat[op.mat];
  const int rows = I.len[op.len];
  const int nd = op.k, off0 = op.b;
  const int cols = c.slen[op.a];
  const double* x = slot_ptr(c, op.a);
  double* y = spare_ptr(c);
  const int total = c_tb * c_lcap;
  constexpr int kU = KU > 2 ? 2 : KU;  // the matrix loads of kU rows before their stores
  for (int base = c_tid; base < total; base += kU * c_nthreads) {
    double acc[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int idx = base + u * c_nthreads;
      acc[u] = 0.0;
      if (idx < total) {
        const int t = idx / c_lcap, r = idx - t * c_lcap;
        if (r < rows) {
          const double* xl = x + t * c_lcap;
          for (int d = 0; d < nd; ++d) {
            const int col = r + off0 + 2 * d;
            if (col >= 0 && col < cols) acc[u] = fma(__ldg(A + d * rows + r), xl[col], acc[u]);
          }
        }
      }
    }
#pragma unroll
    for (int u = 0; u < kU; ++u)
      if (base + u * c_nthreads < total) y[base + u * c_nthreads] = acc[u];
  }
  swap_spare(c, op.a);
  c.slen[op.a] = rows;
}

// D (8x8) += A (8x4, row-major) B (4x8, column-major) on the FP64 tensor cores; per lane
// (g = lane / 4, q = lane % 4): a = A[g][q], b = B[q][g], d0, d1 = D[g][2q], D[g][2q+1].
__device__ __forceinline__ void dmma_8x8x4(double& d0, double& d1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
               : "+d"(d0), "+d"(d1)
               : "d"(a), "d"(b));
}

// y = A x per line on the tensor cores: Y (rows x tb) = A (rows x cols) X (cols x tb), one warp per
// 8-row x 8-line output block, two accumulators over alternating column quads.
__device__ void op_dense_mma(Ctx& c, const pgx_op& op, const pgx_instance& I) {
  const int c_tb = c.tb;
  const int c_lcap = c.lcap;
  const int c_nthreads = c.nthreads;
  const int c_tid = c.tid;
  const double* A = I.mat[op.mat];
  const int rows = I.len[op.len];
  const int cols = c.slen[op.a];
  const double* x = slot_ptr(c, op.a);
  double* y = spare_ptr(c);
  zero_tail(c, y, rows);
  const int lane = c_tid & 31, warp = c_tid >> 5, nw = c_nthreads >> 5;
  const int g = lane >> 2, q = lane & 3;
  const int nrb = (rows + 7) >> 3, nlb = (c_tb + 7) >> 3;
  for (int blk = warp; blk < nrb * nlb; blk += nw) {  // warp-uniform loop
    const int lb = blk / nrb, rb = blk - lb * nrb;
    const int r = rb * 8 + g, t = lb * 8 + g;          // the A row / X line this lane loads
    const bool rok = r < rows, tok = t < c_tb;
    const double* Ar = A + (size_t)(rok ? r : 0) * cols;
    const double* xl = x + (tok ? t : 0) * c_lcap;
    double d0 = 0.0, d1 = 0.0, e0 = 0.0, e1 = 0.0;
    int k = 0;
    for (; k + 8 <= cols; k += 8) {
      const double a0 = rok ? __ldg(Ar + k + q) : 0.0, b0 = tok ? xl[k + q] : 0.0;
      const double a1 = rok ? __ldg(Ar + k + 4 + q) : 0.0, b1 = tok ? xl[k + 4 + q] : 0.0;
      dmma_8x8x4(d0, d1, a0, b0);
      dmma_8x8x4(e0, e1, a1, b1);
    }
    for (; k < cols; k += 4) {
      const bool kok = k + q < cols;
      const double a0 = (rok && kok) ? __ldg(Ar + k + q) : 0.0, b0 = (tok && kok) ? xl[k + q] : 0.0;
      dmma_8x8x4(d0, d1, a0, b0);
    }
    const int orow = rb * 8 + g, t0 = lb * 8 + 2 * q;
    if (orow < rows) {
      if (t0 < c_tb) y[t0 * c_lcap + orow] = d0 + e0;
      if (t0 + 1 < c_tb) y[(t0 + 1) * c_lcap + orow] = d1 + e1;
    }
  }
  __syncthreads();
  swap_spare(c, op.a);
  c.slen[op.a] = rows;
}

__device__ void op_dense(Ctx& c, const pgx_op& op, const pgx_instance& I) {
  const int c_tb = c.tb;
  const int c_lcap = c.lcap;
  const int c_nthreads = c.nthreads;
  const int c_tid = c.tid;
  if (op.k & PGX_DENSE_MMA) {
    op_dense_mma(c, op, I);
    return;
  }
  const double* A = I.mat[op.mat];
  const int rows = I.len[op.len];
  const int cols = c.slen[op.a];
  const double* x = slot_ptr(c, op.a);
  double* y = spare_ptr(c);
  zero_tail(c, y, rows);
  for (int idx = c_tid; idx < c_tb * rows; idx += c_nthreads) {
    int r = idx / c_tb, t = idx - r * c_tb;
    const double* xl = x + t * c_lcap;
    const double* Ar = A + (size_t)r * cols;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    int k = 0;
    for (; k + 3 < cols; k += 4) {
      a0 = fma(__ldg(Ar + k), xl[k], a0);
      a1 = fma(__ldg(Ar + k + 1), xl[k + 1], a1);
      a2 = fma(__ldg(Ar + k + 2), xl[k + 2], a2);
      a3 = fma(__ldg(Ar + k + 3), xl[k + 3], a3);
    }
    for (; k < cols; ++k) a0 = fma(__ldg(Ar + k), xl[k], a0);
    y[t * c_lcap + r] = (a0 + a1) + (a2 + a3);
  }
  __syncthreads();
  swap_spare(c, op.a);
  c.slen[op.a] = rows;
}

// ---------------------------------------------------------------- DCT-I
// DCT-I of two real lines at once: the even extensions e, e' (length L = 2(n-1))
// form z = e + i e'; its DFT Z is y + i y' because the DFT of a real even
// sequence is real.  The complex DFT is a mixed-radix (4, 2, 3) Stockham FFT in
// shared memory; tw[k] = exp(-2 pi i k / L) comes from a host-built table (followed, for the folded
// even transform, by the fold coefficients 1/2 - sin(pi m / N), m < N = L / 2).
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
// p + w q and 2 p - z, each component one or two fused multiply-adds
__device__ __forceinline__ double2 cmadd(double2 p, double2 w, double2 q) {
  return make_double2(fma(w.x, q.x, fma(-w.y, q.y, p.x)), fma(w.x, q.y, fma(w.y, q.x, p.y)));
}
__device__ __forceinline__ double2 ctwice_minus(double2 p, double2 z) {
  return make_double2(fma(2.0, p.x, -z.x), fma(2.0, p.y, -z.y));
}
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }

// Diagonal scalings around the raw DCT-I matrix C (y = post * C (pre * x)), per mode:
//   RAW 1, 1;  FWD 1, m_k (-1)^k / (2N);  BWD (-1)^j / w_j, 1;
//   FWD_T (-1)^j / (2N), w_k;  BWD_T 1 / w_j, (-1)^k   (w = 1 at both ends, 2 inside;
// the transposed modes are the exact adjoints of FWD and BWD because C^T = W C W^-1).
// Every pre-scale is symmetric in j <-> N - j for even N.
// Carried as (mode, 1/N): one division per op, the inner loops only select.
struct DctScale {
  int mode;
  double invN;
  bool has_pre, has_post;
  __device__ __forceinline__ double pre(int j, int N) const {
    const bool end = (j == 0 || j == N);
    const double sg = (j & 1) ? -1.0 : 1.0;
    switch (mode) {
      case PGX_DCT_BWD: return end ? sg : 0.5 * sg;
      case PGX_DCT_FWD_T: return sg * (0.5 * invN);
      case PGX_DCT_BWD_T: return end ? 1.0 : 0.5;
      default: return 1.0;
    }
  }
  // u * pre(j, N), bit for bit; the +-1/2 and 1 of BWD and BWD_T on the bit pattern (no FP64 instruction)
  __device__ __forceinline__ double scale_pre(double u, int j, int N) const {
    const bool end = (j == 0 || j == N);
    switch (mode) {
      case PGX_DCT_BWD: return end ? ((j & 1) ? -u : u) : pgx_half_signed(u, (j & 1) != 0);
      case PGX_DCT_BWD_T: return end ? u : pgx_half_signed(u, false);
      case PGX_DCT_FWD_T: return u * pre(j, N);
      default: return u;
    }
  }
  __device__ __forceinline__ double post(int k, int N) const {
    const bool end = (k == 0 || k == N);
    const double sg = (k & 1) ? -1.0 : 1.0;
    switch (mode) {
      case PGX_DCT_FWD: return sg * (end ? 0.5 * invN : invN);
      case PGX_DCT_FWD_T: return end ? 1.0 : 2.0;
      case PGX_DCT_BWD_T: return sg;
      default: return 1.0;
    }
  }
};
__device__ __forceinline__ DctScale dct_scale(int mode, int N) {
  DctScale s;
  s.mode = mode;
  s.invN = 1.0 / N;
  s.has_pre = mode == PGX_DCT_BWD || mode == PGX_DCT_FWD_T || mode == PGX_DCT_BWD_T;
  s.has_post = mode == PGX_DCT_FWD || mode == PGX_DCT_FWD_T || mode == PGX_DCT_BWD_T;
  return s;
}

// One radix-R Stockham stage over `npairs` pairs of lines.
//   FIRST: the input is the even extension of slot lines (2p, 2p+1), read straight
//          from the slot with the backward pre-scale folded in (no copy pass);
//   LAST:  outputs k <= N are written straight back to the slot lines with the
//          forward post-scale (no extraction pass).
template <int R, bool FIRST, bool LAST>
__device__ __forceinline__ void stockham_stage(const Ctx& c, const double2* src, double2* dst, const double2* tw,
                                               int L, int Ns, int npairs, double* x, const DctScale& ds,
                                               int tws = 1) {
  const int c_tb = c.tb;
  const int c_lcap = c.lcap;
  const int c_nthreads = c.nthreads;
  const int c_tid = c.tid;
  const int c_fft_stride = c.fft_stride;
  const int LR = L / R;
  const int step = tws * (L / (Ns * R));  // twiddle table holds exp(-2 pi i k / (tws L))
  const int N = L >> 1;
  for (int idx = c_tid; idx < npairs * LR; idx += c_nthreads) {
    int pr = idx / LR, j = idx - pr * LR;
    const int t0 = 2 * pr;
    const bool two = t0 + 1 < c_tb;
    int k = j % Ns;
    double2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int m = j + r * LR;
      if (FIRST) {
        const int sidx = m <= N ? m : L - m;
        double a = x[t0 * c_lcap + sidx];
        double b = two ? x[(t0 + 1) * c_lcap + sidx] : 0.0;
        if (ds.has_pre) {
          a = ds.scale_pre(a, sidx, N);
          b = ds.scale_pre(b, sidx, N);
        }
        v[r] = make_double2(a, b);
      } else {
        v[r] = src[pr * c_fft_stride + m];
      }
    }
    double2 o[R];
    if (R != 3 && Ns > 1 && !FIRST && !LAST) {
      // Twiddled radix-2 / radix-4 butterflies as fused multiply-adds (w2 = w1^2, w3 = w1 w2):
      //   a = v0 + w2 v2, b = 2 v0 - a, c = v1 + w2 v3, d = 2 v1 - c,
      //   o0 = a + w1 c, o2 = 2a - o0, o1 = b + (-i w1) d, o3 = 2b - o1
      // (24 FP64 instructions against 28 for three complex products and eight sums).
      const double2 w1 = __ldg(tw + k * step);
      if (R == 2) {
        o[0] = cmadd(v[0], w1, v[1]);
        o[1] = ctwice_minus(v[0], o[0]);
      } else {
        const double2 w2 = __ldg(tw + 2 * k * step);
        const double2 a = cmadd(v[0], w2, v[2]), b = ctwice_minus(v[0], a);
        const double2 cc = cmadd(v[1], w2, v[3]), d = ctwice_minus(v[1], cc);
        o[0] = cmadd(a, w1, cc);
        o[2] = ctwice_minus(a, o[0]);
        o[1] = cmadd(b, make_double2(w1.y, -w1.x), d);
        o[3] = ctwice_minus(b, o[1]);
      }
    } else {
    if (k != 0) {
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], __ldg(tw + k * r * step));
    }
    if (R == 2) {
      o[0] = cadd(v[0], v[1]);
      o[1] = csub(v[0], v[1]);
    } else if (R == 4) {
      double2 a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
      double2 e = cadd(v[1], v[3]), f = csub(v[1], v[3]);
      o[0] = cadd(a, e);
      o[2] = csub(a, e);
      o[1] = make_double2(b.x + f.y, b.y - f.x);  // b - i f
      o[3] = make_double2(b.x - f.y, b.y + f.x);  // b + i f
    } else {  // R == 3, W3 = -1/2 - i sqrt(3)/2
      const double h = 0.86602540378443864676;
      double2 t1 = cadd(v[1], v[2]);
      double2 t2 = make_double2(fma(-0.5, t1.x, v[0].x), fma(-0.5, t1.y, v[0].y));
      double2 t3 = csub(v[1], v[2]);
      o[0] = cadd(v[0], t1);
      o[1] = make_double2(fma(h, t3.y, t2.x), fma(-h, t3.x, t2.y));  // t2 - i h t3
      o[2] = make_double2(fma(-h, t3.y, t2.x), fma(h, t3.x, t2.y));  // t2 + i h t3
    }
    }
    const int base = (j - k) * R + k;
#pragma unroll
    for (int q = 0; q < R; ++q) {
      const int kk = base + q * Ns;
      if (LAST) {
        if (kk <= N) {
          double2 z = o[q];
          if (ds.has_post) {
            const double sc = ds.post(kk, N);
            z.x *= sc;
            z.y *= sc;
          }
          x[t0 * c_lcap + kk] = z.x;
          if (two) x[(t0 + 1) * c_lcap + kk] = z.y;
        }
      } else {
        dst[pr * c_fft_stride + kk] = o[q];
      }
    }
  }
}

__device__ __forceinline__ void x_nan(const Ctx& c, int slot, int idx, int n) {
  int t = idx / n, k = idx - t * n;
  slot_ptr(c, slot)[t * c.lcap + k] = __longlong_as_double(0x7ff8000000000000ULL);
}

__device__ __forceinline__ int next_radix(int rem) { return (rem & 3) == 0 ? 4 : ((rem & 1) == 0 ? 2 : 3); }

template <bool FIRST, bool LAST>
__device__ __forceinline__ void stage_dispatch(int R, const Ctx& c, const double2* src, double2* dst, const double2* tw,
                                               int L, int Ns, int npairs, double* x, const DctScale& ds,
                                               int tws = 1) {
  if (R == 4) stockham_stage<4, FIRST, LAST>(c, src, dst, tw, L, Ns, npairs, x, ds, tws);
  else if (R == 2) stockham_stage<2, FIRST, LAST>(c, src, dst, tw, L, Ns, npairs, x, ds, tws);
  else stockham_stage<3, FIRST, LAST>(c, src, dst, tw, L, Ns, npairs, x, ds, tws);
}

// Radix plan of the length-N FFT: every factor 3 first (the first stage has no twiddles, and a
// twiddled radix-3 stage costs the most FP64 instructions per point), then 4s, then one 2.
struct RadixPlan {
  int n3, n4, n2;  // stages of radix 3, then 4, then 2
  __device__ __forceinline__ int stages() const { return n3 + n4 + n2; }
  __device__ __forceinline__ int at(int s) const { return s < n3 ? 3 : (s < n3 + n4 ? 4 : 2); }
};
__device__ __forceinline__ RadixPlan radix_plan(int N, int& rest, bool radix2 = false) {
  RadixPlan p{0, 0, 0};
  int m = N;
  while (m % 3 == 0) { ++p.n3; m /= 3; }
  if (radix2) {
    while (m % 2 == 0) { ++p.n2; m /= 2; }
  } else {
    while (m % 4 == 0) { ++p.n4; m /= 4; }
    if (m % 2 == 0) { ++p.n2; m /= 2; }
  }
  rest = m;  // 1 for every length with a twiddle table (n - 1 = 2^a 3^b)
  return p;
}

// The plan with an odd number of stages, for a transform that ping-pongs between the slot and the
// spare (the first stage reads the slot and writes the spare, so the last one writes the spare
// too): one radix-4 stage split into two radix-2 stages (the same FP64 instructions per point), or
// two radix-2 stages merged; no stages when neither exists (N = 2 * 3^b with b odd).
__device__ __forceinline__ RadixPlan odd_stages(RadixPlan p) {
  if (p.stages() & 1) return p;
  if (p.n4 > 0) return RadixPlan{p.n3, p.n4 - 1, p.n2 + 2};
  if (p.n2 >= 2) return RadixPlan{p.n3, p.n4 + 1, p.n2 - 2};
  return RadixPlan{0, 0, 0};
}

// Untwiddled radix-R butterfly (the first stage of an FFT).
template <int R>
__device__ __forceinline__ void butterfly_plain(double2* v, double2* o) {
  if (R == 2) {
    o[0] = cadd(v[0], v[1]);
    o[1] = csub(v[0], v[1]);
  } else if (R == 4) {
    double2 a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
    double2 e = cadd(v[1], v[3]), f = csub(v[1], v[3]);
    o[0] = cadd(a, e);
    o[2] = csub(a, e);
    o[1] = make_double2(b.x + f.y, b.y - f.x);  // b - i f
    o[3] = make_double2(b.x - f.y, b.y + f.x);  // b + i f
  } else {  // R == 3, W3 = -1/2 - i sqrt(3)/2
    const double h = 0.86602540378443864676;
    double2 t1 = cadd(v[1], v[2]);
    double2 t2 = make_double2(fma(-0.5, t1.x, v[0].x), fma(-0.5, t1.y, v[0].y));
    double2 t3 = csub(v[1], v[2]);
    o[0] = cadd(v[0], t1);
    o[1] = make_double2(fma(h, t3.y, t2.x), fma(-h, t3.x, t2.y));  // t2 - i h t3
    o[2] = make_double2(fma(-h, t3.y, t2.x), fma(h, t3.x, t2.y));  // t2 + i h t3
  }
}

// The first radix-R stage of the even DCT's FFT (Ns = 1, no twiddles) with the fold computed on
// its way in: u_m = (x_m + x_{N-m})/2 - sin(pi m/N) (x_m - x_{N-m}) = x_{N-m} + (1/2 - sin(pi m/N))
// (x_m - x_{N-m}), one FMA a point, of both lines of every pair, read straight from the slots (no
// separate fold phase, one barrier fewer per transform).
template <int R>
__device__ __forceinline__ void fold_stage(const Ctx& c, double2* dst, const double2* tw, int N, int nall,
                                           int npairs, int slot0, const DctScale& ds) {
  const int c_tb = c.tb;
  const int c_lcap = c.lcap;
  const int c_nthreads = c.nthreads;
  const int c_tid = c.tid;
  const int c_fft_stride = c.fft_stride;
  const int LR = N / R;
  const double* cmt = reinterpret_cast<const double*>(tw + 2 * N);
  double* const x0s = slot_ptr(c, slot0);
  for (int idx = c_tid; idx < nall * LR; idx += c_nthreads) {
    const int P = idx / LR, j = idx - P * LR;
    const int sl = P / npairs, pr = P - sl * npairs;
    const double* x = op_slot(c, x0s, slot0, sl);
    const int t0 = 2 * pr;
    const bool two = t0 + 1 < c_tb;
    double2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int m = j + r * LR;
      const double cm = __ldg(cmt + m);  // 1/2 - sin(pi m / N), after the 2N twiddles
      const double a0 = x[t0 * c_lcap + m], a1 = x[t0 * c_lcap + N - m];
      double ua = fma(cm, a0 - a1, a1);
      double ub = 0.0;
      if (two) {
        const double b0 = x[(t0 + 1) * c_lcap + m], b1 = x[(t0 + 1) * c_lcap + N - m];
        ub = fma(cm, b0 - b1, b1);
      }
      if (ds.has_pre) {
        ua = ds.scale_pre(ua, m, N);
        ub = ds.scale_pre(ub, m, N);
      }
      v[r] = make_double2(ua, ub);
    }
    double2 o[R];
    butterfly_plain<R>(v, o);
#pragma unroll
    for (int q = 0; q < R; ++q) dst[P * c_fft_stride + j * R + q] = o[q];
  }
}

// DCT-I for even N = n - 1, exploiting both the realness and the even symmetry
// of the extension (half the FFT length of the paired approach):
//   fold   u_j = (x_j + x_{N-j})/2 - sin(pi j/N) (x_j - x_{N-j}),  j = 0..N-1
//          y_1 = (x_0 - x_N) + 2 sum_{0<j<N/2} (x_j - x_{N-j}) cos(pi j/N)
//   FFT    Z = DFT_N(u_a + i u_b) for the two lines (a, b) of a pair
//   untangle  y_{2m} = Z_m + conj(Z_{N-m}) (real / imag part for line a / b),
//          odd increments y_{2m+1} - y_{2m-1} = Im(Z_{N-m} - Z_m) (a), Re(Z_m - Z_{N-m}) (b)
//   scan   y_{2m+1} = y_1 + sum of increments.
// Every phase runs over all threads of the CTA (a barrier between phases), with the FFT's radix
// plan (radix_plan), the fold and the per-line phases (L lanes a line) of the warp-local form.
// tw is the table exp(-2 pi i k / (2N)): W_N^k = tw[2k], (cos, -sin)(pi j / N) = tw[j].
// The backward pre-scale (-1)^j w_j is common to x_j and x_{N-j} (N even) and
// applied to u_j, d_j; the forward post-scale to the outputs.
__device__ void op_dct_even_cta(Ctx& c, const pgx_op& op, const pgx_instance& I) {
  const int c_tb = c.tb;
  const int c_lcap = c.lcap;
  const int c_nthreads = c.nthreads;
  const int c_tid = c.tid;
  const int c_fft_stride = c.fft_stride;
  double* const c_ybuf = c.ybuf;
  // op.b > 1: the transforms of slots a .. a+b-1 (same length and mode) go through every
  // phase together: one barrier per phase for all of them, b times the parallel work.
  const int ns = nslot_of(op);
  double* const x0s = slot_ptr(c, op.a);
  const int n = c.slen[op.a];
  const int N = n - 1, H = N / 2;
  const int mode = op.k & PGX_DCT_MODE_MASK;
  const DctScale ds = dct_scale(mode, N);
  const double2* tw = reinterpret_cast<const double2*>(I.mat[op.mat]);
  const int npairs = (c_tb + 1) >> 1;
  const int nall = ns * npairs;  // line pairs of all slots; pair P = s * npairs + pr
  int rest = 1;
  const bool in_slot = (op.k & PGX_DCT_SLOT) != 0;
  const RadixPlan plan = in_slot ? odd_stages(radix_plan(N, rest)) : radix_plan(N, rest);
  if (N > c_fft_stride || rest != 1 || plan.stages() < 1 || (in_slot && (ns != 1 || (c_tb & 1)))) {
    // no buffer or plan for this length: refuse loudly
    for (int sl = 0; sl < ns; ++sl)
      for (int idx = c_tid; idx < c_tb * n; idx += c_nthreads) x_nan(c, op.a + sl, idx, n);
    return;
  }
  // y_1, L lanes a line, the op's lines spread over the warps (line lt = sl * tb + t); the j of a
  // lane keep one parity (L even), so the alternating pre-scale of BWD / FWD_T is one sign per lane
  const int nlines = ns * c_tb;
  const LineLanes g = line_lanes(c, nlines);
  {
    const bool alt = mode == PGX_DCT_BWD || mode == PGX_DCT_FWD_T;
    const double ps = ds.has_pre ? (alt ? -ds.pre(1, N) : ds.pre(1, N)) : 1.0;
    const double p0 = ds.has_pre ? ds.pre(0, N) : 1.0;
    for (int base = g.first; base < nlines; base += g.stride) {
      const int lt = base + g.grp;
      const bool valid = lt < nlines;
      const int sl = valid ? lt / c_tb : 0, t = valid ? lt - sl * c_tb : 0;
      const double* xl = op_slot(c, x0s, op.a, sl) + t * c_lcap;
      double acc = 0.0;
      if (valid)
        for (int j = 1 + g.sub; j < H; j += g.L) acc = fma(__ldg(&tw[j].x), xl[j] - xl[N - j], acc);
      if (alt && ((1 + g.sub) & 1)) acc = -acc;
      for (int o = g.L >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, g.L);
      if (valid && g.sub == 0) c_ybuf[lt] = fma(2.0 * ps, acc, (xl[0] - xl[N]) * p0);
    }
  }
  // FFT of length N over all pairs, the radix plan of the warp-local form (y_1 above and the first
  // stage both only read the slots)
  double2* bufs[2] = {c.f0, c.f1};
  const int R0 = plan.at(0);
  if (R0 == 3) fold_stage<3>(c, bufs[1], tw, N, nall, npairs, op.a, ds);
  else if (R0 == 4) fold_stage<4>(c, bufs[1], tw, N, nall, npairs, op.a, ds);
  else fold_stage<2>(c, bufs[1], tw, N, nall, npairs, op.a, ds);
  int cur = 1, Ns = R0;
  for (int s = 1; s < plan.stages(); ++s) {
    __syncthreads();
    stage_dispatch<false, false>(plan.at(s), c, bufs[cur], bufs[cur ^ 1], tw, N, Ns, nall, nullptr, ds, 2);
    cur ^= 1;
    Ns *= plan.at(s);
  }
  __syncthreads();
  const double2* Z = bufs[cur];
  // untangle: even outputs, odd increments
  for (int idx = c_tid; idx < nall * (H + 1); idx += c_nthreads) {
    const int P = idx / (H + 1), m = idx - P * (H + 1);
    const int sl = P / npairs, pr = P - sl * npairs;
    double* x = op_slot(c, x0s, op.a, sl);
    const int t0 = 2 * pr;
    const bool two = t0 + 1 < c_tb;
    const double2 zm = Z[P * c_fft_stride + m];
    const double2 zn = Z[P * c_fft_stride + (m == 0 ? 0 : N - m)];
    double ya = zm.x + zn.x, yb = zm.y + zn.y;
    if (ds.has_post) {
      const double sc = ds.post(2 * m, N);
      ya *= sc;
      yb *= sc;
    }
    x[t0 * c_lcap + 2 * m] = ya;
    if (two) x[(t0 + 1) * c_lcap + 2 * m] = yb;
    if (m >= 1 && m < H) {
      x[t0 * c_lcap + 2 * m + 1] = zn.y - zm.y;
      if (two) x[(t0 + 1) * c_lcap + 2 * m + 1] = zm.x - zn.x;
    } else if (m == 0) {
      x[t0 * c_lcap + 1] = c_ybuf[sl * c_tb + t0];
      if (two) x[(t0 + 1) * c_lcap + 1] = c_ybuf[sl * c_tb + t0 + 1];
    }
  }
  if (in_slot) zero_tail(c, slot_ptr(c, op.a), n);  // the FFT stages wrote past the lines' ends
  __syncthreads();
  // odd outputs: inclusive prefix sums over k = 1, 3, ..., N-1, L lanes a line
  {
    const int chunk = (H + g.L - 1) / g.L;
    const double osc = ds.has_post ? ds.post(1, N) : 1.0;  // the same for every odd k < N
    for (int base = g.first; base < nlines; base += g.stride) {
      const int lt = base + g.grp;
      const bool valid = lt < nlines;
      const int sl = valid ? lt / c_tb : 0, t = valid ? lt - sl * c_tb : 0;
      double* xl = op_slot(c, x0s, op.a, sl) + t * c_lcap;
      const int m0 = min(g.sub * chunk, H), m1 = min(m0 + chunk, H);
      double run = 0.0;
      if (valid)
        for (int m = m0; m < m1; ++m) run += xl[2 * m + 1];
      double incl = run;
      for (int o = 1; o < g.L; o <<= 1) {
        const double v = __shfl_up_sync(0xffffffffu, incl, o, g.L);
        if (g.sub >= o) incl += v;
      }
      if (!valid) continue;
      double pre = incl - run;  // exclusive prefix of this lane's chunk
      if (ds.has_post) {
        for (int m = m0; m < m1; ++m) {
          pre += xl[2 * m + 1];
          xl[2 * m + 1] = pre * osc;
        }
      } else {
        for (int m = m0; m < m1; ++m) {
          pre += xl[2 * m + 1];
          xl[2 * m + 1] = pre;
        }
      }
    }
  }
}

// ---------------------------------------------------------- warp-local even DCT
// The same folded half-length algorithm as op_dct_even_cta, with every phase of a line pair
// inside one warp: warp w owns the pairs P = w, w + nw, w + 2 nw, ... of all the op's slots and
// runs their fold, FFT stages, untangle and scan separated by __syncwarp only, so the warps of a
// CTA (and of the other CTAs on the SM) never wait for each other inside a transform.  Per line,
// y_1 and the odd-coefficient scan use just enough lanes to cover the warp's lines (L lanes a
// line, log2 L shuffle steps instead of 32 lanes and 5), and the fold is one FMA per point:
// u_m = (x_m + x_{N-m})/2 - sin(pi m/N) (x_m - x_{N-m}) = x_{N-m} + (1/2 - sin(pi m/N)) (x_m - x_{N-m}).

struct WarpPairs {
  int lane, w, nw, npw;  // lane, warp, warps of the CTA, pairs this warp owns
};
__device__ __forceinline__ WarpPairs warp_pairs(const Ctx& c, int nall) {
  WarpPairs g;
  g.lane = c.tid & 31;
  g.w = c.tid >> 5;
  g.nw = c.nthreads >> 5;
  g.npw = g.w < nall ? (nall - g.w + g.nw - 1) / g.nw : 0;
  return g;
}

// First stage (Ns = 1, no twiddles) with the fold on its way in, over the warp's pairs.
template <int R>
__device__ __forceinline__ void wfold(const Ctx& c, const WarpPairs& g, double2* dst, const double2* tw, int N,
                                      int npairs, int slot0, const DctScale& ds) {
  const int c_tb = c.tb;
  const int c_lcap = c.lcap;
  const int c_fft_stride = c.fft_stride;
  const int B = N / R;
  const double* cmt = reinterpret_cast<const double*>(tw + 2 * N);
  double* const x0s = slot_ptr(c, slot0);
  for (int it = g.lane; it < g.npw * B; it += 32) {
    const int q = it / B, j = it - q * B;
    const int P = g.w + q * g.nw;
    const int sl = P / npairs, pr = P - sl * npairs;
    const double* x = op_slot(c, x0s, slot0, sl);
    const int t0 = 2 * pr;
    const bool two = t0 + 1 < c_tb;
    double2 v[R], o[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int m = j + r * B;
      const double cm = __ldg(cmt + m);  // 1/2 - sin(pi m / N), after the 2N twiddles
      const double a0 = x[t0 * c_lcap + m], a1 = x[t0 * c_lcap + N - m];
      double ua = fma(cm, a0 - a1, a1);
      double ub = 0.0;
      if (two) {
        const double b0 = x[(t0 + 1) * c_lcap + m], b1 = x[(t0 + 1) * c_lcap + N - m];
        ub = fma(cm, b0 - b1, b1);
      }
      if (ds.has_pre) {
        ua = ds.scale_pre(ua, m, N);
        ub = ds.scale_pre(ub, m, N);
      }
      v[r] = make_double2(ua, ub);
    }
    butterfly_plain<R>(v, o);
#pragma unroll
    for (int q2 = 0; q2 < R; ++q2) dst[P * c_fft_stride + j * R + q2] = o[q2];
  }
}

// One twiddled radix-R Stockham stage (Ns > 1) over the warp's pairs; tw holds exp(-2 pi i k / (tws L)).
template <int R>
__device__ __forceinline__ void wstage(const Ctx& c, const WarpPairs& g, const double2* src, double2* dst,
                                       const double2* tw, int L, int Ns, int tws) {
  const int c_fft_stride = c.fft_stride;
  const int B = L / R;
  const int step = tws * (L / (Ns * R));
  for (int it = g.lane; it < g.npw * B; it += 32) {
    const int q = it / B, j = it - q * B;
    const int P = g.w + q * g.nw;
    const int k = j % Ns;
    const double2* s = src + P * c_fft_stride;
    double2 v[R], o[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = s[j + r * B];
    if (R == 2) {
      const double2 w1 = __ldg(tw + k * step);
      o[0] = cmadd(v[0], w1, v[1]);
      o[1] = ctwice_minus(v[0], o[0]);
    } else if (R == 4) {
      const double2 w1 = __ldg(tw + k * step), w2 = __ldg(tw + 2 * k * step);
      const double2 a = cmadd(v[0], w2, v[2]), b = ctwice_minus(v[0], a);
      const double2 cc = cmadd(v[1], w2, v[3]), d = ctwice_minus(v[1], cc);
      o[0] = cmadd(a, w1, cc);
      o[2] = ctwice_minus(a, o[0]);
      o[1] = cmadd(b, make_double2(w1.y, -w1.x), d);
      o[3] = ctwice_minus(b, o[1]);
    } else {
      if (k != 0) {
        v[1] = cmul(v[1], __ldg(tw + k * step));
        v[2] = cmul(v[2], __ldg(tw + 2 * k * step));
      }
      butterfly_plain<3>(v, o);
    }
    double2* d = dst + P * c_fft_stride + (j - k) * R + k;
#pragma unroll
    for (int q2 = 0; q2 < R; ++q2) d[q2 * Ns] = o[q2];
  }
}

__device__ void op_dct_even(Ctx& c, const pgx_op& op, const pgx_instance& I) {
  const int c_tb = c.tb;
  const int c_lcap = c.lcap;
  const int c_nthreads = c.nthreads;
  const int c_tid = c.tid;
  const int c_fft_stride = c.fft_stride;
  double* const c_ybuf = c.ybuf;
  const int ns = nslot_of(op);
  double* const x0s = slot_ptr(c, op.a);
  const int n = c.slen[op.a];
  const int N = n - 1, H = N / 2;
  const int mode = op.k & PGX_DCT_MODE_MASK;
  const DctScale ds = dct_scale(mode, N);
  const double2* tw = reinterpret_cast<const double2*>(I.mat[op.mat]);
  const int npairs = (c_tb + 1) >> 1;
  const int nall = ns * npairs;  // line pairs of all slots; pair P = s * npairs + pr
  int rest = 1;
  const bool in_slot = (op.k & PGX_DCT_SLOT) != 0;
  const RadixPlan plan = radix_plan(N, rest);
  if (N > c_fft_stride || rest != 1 || plan.stages() < 1 ||
      (in_slot && (ns != 1 || (c_tb & 1) || odd_stages(plan).stages() < 1))) {
    // no buffer or plan for this length: refuse loudly
    for (int sl = 0; sl < ns; ++sl)
      for (int idx = c_tid; idx < c_tb * n; idx += c_nthreads) x_nan(c, op.a + sl, idx, n);
    return;
  }
  const WarpPairs g = warp_pairs(c, nall);
  if (g.npw == 0) return;
  // A radix-4 stage and two radix-2 stages issue the same FP64 instructions per point, but the
  // warp's butterfly count per stage (npw N / R) leaves different numbers of lanes idle in its last
  // iteration: take radix 2 where that needs fewer FP64 warp instructions (6 per radix-2 butterfly
  // and level, 24 per radix-4 butterfly and two levels).
  RadixPlan wplan = 6 * ((g.npw * N + 63) >> 6) < 12 * ((g.npw * N + 127) >> 7) ? radix_plan(N, rest, true) : plan;
  if (in_slot) wplan = odd_stages(wplan);  // the last stage writes the spare, not the slot
  const int nl = 2 * g.npw;  // lines of the warp's pairs (the last one of an odd tile may not exist)
  const int L = lanes_per_line(nl), per = 32 / L, grp = g.lane / L, sub = g.lane & (L - 1);

  // y_1, L lanes a line: the j of a lane keep one parity (L even), so the alternating pre-scale
  // of BWD / FWD_T is one sign per lane
  {
    const bool alt = mode == PGX_DCT_BWD || mode == PGX_DCT_FWD_T;
    const double ps = ds.has_pre ? (alt ? -ds.pre(1, N) : ds.pre(1, N)) : 1.0;
    const double p0 = ds.has_pre ? ds.pre(0, N) : 1.0;
    for (int base = 0; base < nl; base += per) {
      const int ll = base + grp, q = ll >> 1;
      const int P = g.w + q * g.nw;
      const int sl = P / npairs, t = 2 * (P - sl * npairs) + (ll & 1);
      const bool valid = ll < nl && t < c_tb;
      double acc = 0.0;
      const double* xl = op_slot(c, x0s, op.a, valid ? sl : 0) + (valid ? t : 0) * c_lcap;
      if (valid)
        for (int j = 1 + sub; j < H; j += L) acc = fma(__ldg(&tw[j].x), xl[j] - xl[N - j], acc);
      if (alt && ((1 + sub) & 1)) acc = -acc;
      for (int o = L >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, L);
      if (valid && sub == 0) c_ybuf[sl * c_tb + t] = fma(2.0 * ps, acc, (xl[0] - xl[N]) * p0);
    }
  }
  // FFT of length N over the warp's pairs, ping-pong between the two buffers
  double2* bufs[2] = {c.f0, c.f1};
  const int R0 = wplan.at(0);
  if (R0 == 3) wfold<3>(c, g, bufs[1], tw, N, npairs, op.a, ds);
  else if (R0 == 4) wfold<4>(c, g, bufs[1], tw, N, npairs, op.a, ds);
  else wfold<2>(c, g, bufs[1], tw, N, npairs, op.a, ds);
  int cur = 1, Ns = R0;
  for (int s = 1; s < wplan.stages(); ++s) {
    __syncwarp();
    const int R = wplan.at(s);
    if (R == 4) wstage<4>(c, g, bufs[cur], bufs[cur ^ 1], tw, N, Ns, 2);
    else if (R == 2) wstage<2>(c, g, bufs[cur], bufs[cur ^ 1], tw, N, Ns, 2);
    else wstage<3>(c, g, bufs[cur], bufs[cur ^ 1], tw, N, Ns, 2);
    cur ^= 1;
    Ns *= R;
  }
  __syncwarp();
  const double2* Z = bufs[cur];
  // untangle: even outputs, odd increments (y_1 from the y_1 phase)
  for (int it = g.lane; it < g.npw * (H + 1); it += 32) {
    const int q = it / (H + 1), m = it - q * (H + 1);
    const int P = g.w + q * g.nw;
    const int sl = P / npairs, pr = P - sl * npairs;
    double* x = op_slot(c, x0s, op.a, sl);
    const int t0 = 2 * pr;
    const bool two = t0 + 1 < c_tb;
    const double2 zm = Z[P * c_fft_stride + m];
    const double2 zn = Z[P * c_fft_stride + (m == 0 ? 0 : N - m)];
    double ya = zm.x + zn.x, yb = zm.y + zn.y;
    if (ds.has_post) {
      const double sc = ds.post(2 * m, N);
      ya *= sc;
      yb *= sc;
    }
    x[t0 * c_lcap + 2 * m] = ya;
    if (two) x[(t0 + 1) * c_lcap + 2 * m] = yb;
    if (m >= 1 && m < H) {
      x[t0 * c_lcap + 2 * m + 1] = zn.y - zm.y;
      if (two) x[(t0 + 1) * c_lcap + 2 * m + 1] = zm.x - zn.x;
    } else if (m == 0) {
      x[t0 * c_lcap + 1] = c_ybuf[sl * c_tb + t0];
      if (two) x[(t0 + 1) * c_lcap + 1] = c_ybuf[sl * c_tb + t0 + 1];
    }
  }
  if (in_slot) {  // the FFT stages wrote past the ends of the warp's lines: zero [n, lcap) again
    const int w = c_lcap - n;
    double* x = slot_ptr(c, op.a);
    for (int it = g.lane; it < g.npw * 2 * w; it += 32) {
      const int q = it / (2 * w), r = it - q * 2 * w;
      const int t = 2 * (g.w + q * g.nw) + (r >= w ? 1 : 0);  // one slot: pair P = line pair P
      x[t * c_lcap + n + (r >= w ? r - w : r)] = 0.0;
    }
  }
  __syncwarp();
  // odd outputs: inclusive prefix sums over k = 1, 3, ..., N-1, L lanes a line
  {
    const int chunk = (H + L - 1) / L;
    const double osc = ds.has_post ? ds.post(1, N) : 1.0;  // the same for every odd k < N
    for (int base = 0; base < nl; base += per) {
      const int ll = base + grp, q = ll >> 1;
      const int P = g.w + q * g.nw;
      const int sl = P / npairs, t = 2 * (P - sl * npairs) + (ll & 1);
      const bool valid = ll < nl && t < c_tb;
      double* xl = op_slot(c, x0s, op.a, valid ? sl : 0) + (valid ? t : 0) * c_lcap;
      const int m0 = min(sub * chunk, H), m1 = min(m0 + chunk, H);
      double run = 0.0;
      if (valid)
        for (int m = m0; m < m1; ++m) run += xl[2 * m + 1];
      double incl = run;
      for (int o = 1; o < L; o <<= 1) {
        const double v = __shfl_up_sync(0xffffffffu, incl, o, L);
        if (sub >= o) incl += v;
      }
      if (!valid) continue;
      double pre = incl - run;  // exclusive prefix of this lane's chunk
      if (ds.has_post) {
        for (int m = m0; m < m1; ++m) {
          pre += xl[2 * m + 1];
          xl[2 * m + 1] = pre * osc;
        }
      } else {
        for (int m = m0; m < m1; ++m) {
          pre += xl[2 * m + 1];
          xl[2 * m + 1] = pre;
        }
      }
    }
  }
}

// DCT-I of the slot (length n) in place: the folded half-length algorithm for
// even n - 1, otherwise paired lines through a length-2(n-1) FFT (stockham_stage).
__device__ void dct_paired_slot(Ctx& c, int slot, const pgx_op& op, const pgx_instance& I);

__device__ void op_dct(Ctx& c, const pgx_op& op, const pgx_instance& I) {
  const int c_tb = c.tb;
  const int c_nthreads = c.nthreads;
  const int c_tid = c.tid;
  const int n = c.slen[op.a];
  if (((n - 1) & 1) == 0 && n >= 3) {
    // a tile with fewer line pairs per slot than warps (single instances, short passes) leaves
    // warps idle in the warp-local form; there the CTA-wide form spreads each pair over all warps
    // (per slot, so a multi-slot op and its one-op-per-slot split take the same form)
    if ((op.k & PGX_DCT_CTA) || ((c_tb + 1) >> 1) < (c_nthreads >> 5)) op_dct_even_cta(c, op, I);
    else op_dct_even(c, op, I);
    return;
  }
  const int ns = nslot_of(op);  // paired-line path: one slot after the other
  if (op.k & PGX_DCT_SLOT) {  // needs 2(n - 1) complex values a pair: no room in the slot, refuse loudly
    for (int sl = 0; sl < ns; ++sl)
      for (int idx = c_tid; idx < c_tb * n; idx += c_nthreads) x_nan(c, op.a + sl, idx, n);
    return;
  }
  for (int sl = 0; sl < ns; ++sl) {
    dct_paired_slot(c, op.a + sl, op, I);
    __syncthreads();
  }
}

__device__ void dct_paired_slot(Ctx& c, int slot, const pgx_op& op, const pgx_instance& I) {
  const int c_tb = c.tb;
  const int c_lcap = c.lcap;
  const int c_nthreads = c.nthreads;
  const int c_tid = c.tid;
  const int c_fft_stride = c.fft_stride;
  const int n = c.slen[slot];
  if (2 * (n - 1) > c_fft_stride) {  // buffer sized for a shorter even length: refuse loudly
    for (int idx = c_tid; idx < c_tb * n; idx += c_nthreads) x_nan(c, slot, idx, n);
    return;
  }
  const int N = n - 1, L = 2 * N;
  const DctScale ds = dct_scale(op.k & PGX_DCT_MODE_MASK, N);
  const double2* tw = reinterpret_cast<const double2*>(I.mat[op.mat]);
  double* x = slot_ptr(c, slot);
  const int npairs = (c_tb + 1) >> 1;
  int nst = 0;
  for (int rem = L; rem > 1; rem /= next_radix(rem)) ++nst;
  double2* bufs[2] = {c.f0, c.f1};
  int Ns = 1, rem = L, cur = 0;
  for (int s = 0; s < nst; ++s) {
    const int R = next_radix(rem);
    const double2* src = bufs[cur];
    double2* dst = bufs[cur ^ 1];
    if (s == 0) {
      if (nst == 1) {
        stage_dispatch<true, false>(R, c, nullptr, c.f0, tw, L, Ns, npairs, x, ds);
      } else {
        stage_dispatch<true, false>(R, c, nullptr, c.f0, tw, L, Ns, npairs, x, ds);
        cur = 0;
        Ns *= R;
        rem /= R;
        __syncthreads();
        continue;
      }
    } else if (s == nst - 1) {
      stage_dispatch<false, true>(R, c, src, nullptr, tw, L, Ns, npairs, x, ds);
    } else {
      stage_dispatch<false, false>(R, c, src, dst, tw, L, Ns, npairs, x, ds);
      cur ^= 1;
    }
    Ns *= R;
    rem /= R;
    __syncthreads();
  }
  if (nst == 1) {  // tiny transform: copy the single stage's output back
    for (int idx = c_tid; idx < c_tb * n; idx += c_nthreads) {
      int t = idx / n, k = idx - t * n;
      double2 z = c.f0[(t >> 1) * c_fft_stride + k];
      double y = (t & 1) ? z.y : z.x;
      if (ds.has_post) y *= ds.post(k, N);
      x[t * c_lcap + k] = y;
    }
  }
}

// ------------------------------------------------------------------ driver
// One tile of one instance: the program's ops on shared-memory slots that start at `sm`.
template <bool FFT, int KU>
__device__ void run_program(const pgx_program& P, const pgx_instance& I, int tile, double* sm) {
  Ctx c;
  c.tb = P.tb;
  c.lcap = P.lcap;
  c.nthreads = blockDim.x;
  c.tid = threadIdx.x;
  c.l0 = tile * P.tb;
  c.nlines = I.len[P.lines_len];
  const int nbuf = P.nslots + 1;
  c.sm = sm;
  size_t off = (size_t)nbuf * c.tb * c.lcap;
  c.fft_stride = pgx_fft_stride(P.fft_n);
  const int fs = pgx_fft_slots(P);
  const bool in_slot = FFT && pgx_fft_in_slot(P);
  const bool fft_in_spare = FFT && !in_slot && pgx_fft_in_spare(P);
  const size_t fbuf = in_slot ? 0 : (size_t)fs * ((c.tb + 1) >> 1) * c.fft_stride;
  double2* const f0 = reinterpret_cast<double2*>(c.sm + off + (off & 1));
  double2* const f1 = fft_in_spare ? nullptr : f0 + fbuf;
  c.ybuf = reinterpret_cast<double*>((fft_in_spare || in_slot ? f0 : f1) + fbuf);
  const int fft_stride = c.fft_stride;
  for (int s = 0; s < nbuf; ++s) c.phys[s] = s;
  for (int s = 0; s < PGX_MAX_SLOTS; ++s) c.slen[s] = 0;
  c.spare = P.nslots;
  for (int s = 0; s < nbuf; ++s) {
    double* b = c.sm + (size_t)s * c.tb * c.lcap;
    for (int i = c.tid; i < c.tb * c.lcap; i += c.nthreads) b[i] = 0.0;
  }
  __syncthreads();
  for (int o = 0; o < P.nops; ++o) {
    const pgx_op& op = P.ops[o];
    switch (op.code) {
      case PGX_OP_LOAD: op_load<KU>(c, op, I, P.axis, 0); break;
      case PGX_OP_LOAD_ADD: op_load<KU>(c, op, I, P.axis, 1); break;
      case PGX_OP_LOAD_MUL: op_load<KU>(c, op, I, P.axis, 2); break;
      case PGX_OP_STORE: op_store<KU>(c, op, I, P.axis, false); break;
      case PGX_OP_STORE_ADD: op_store<KU>(c, op, I, P.axis, true); break;
      case PGX_OP_SCALE:
      case PGX_OP_AXPY:
      case PGX_OP_MUL:
      case PGX_OP_COPY: op_pointwise(c, op, I); break;
      case PGX_OP_SETLEN: op_setlen(c, op, I); break;
      case PGX_OP_STENCIL: op_stencil<KU>(c, op, I); break;
      case PGX_OP_STENCIL_T: op_stencil_t<KU>(c, op, I); break;
      case PGX_OP_TDMA2: op_tdma2(c, op, I); break;
      case PGX_OP_DIFF: op_diff(c, op); break;
      case PGX_OP_DCT:
        if (FFT) {  // programs with DCT ops run the FFT kernels only
          if (op.k & PGX_DCT_SLOT) {  // ping-pong between the slot's own line pairs and the spare
            c.f0 = reinterpret_cast<double2*>(slot_ptr(c, op.a));  // even tb: 16-byte aligned
            c.f1 = reinterpret_cast<double2*>(spare_ptr(c));
            c.fft_stride = c.lcap;  // a pair's two lines, in complex elements
          } else {
            c.f0 = in_slot ? nullptr : f0;
            c.f1 = fft_in_spare ? reinterpret_cast<double2*>(spare_ptr(c)) : f1;
            c.fft_stride = in_slot ? 0 : fft_stride;
          }
          op_dct(c, op, I);
        }
        break;
      case PGX_OP_BANDED: op_banded<KU>(c, op, I); break;
      case PGX_OP_DENSE: op_dense(c, op, I); break;
      case PGX_OP_FDMA: op_fdma(c, op, I, false); break;
      case PGX_OP_POISSON: op_fdma(c, op, I, true); break;
      case PGX_OP_DIFF_T: op_diff_t(c, op); break;
      case PGX_OP_FDMA_T: op_fdma(c, op, I, false, true); break;
      case PGX_OP_POISSON_T: op_fdma(c, op, I, true, true); break;
      case PGX_OP_ZERO00:
        if (c.l0 == 0 && c.tid == 0) slot_ptr(c, op.a)[0] = 0.0;
        break;
      default: break;
    }
    __syncthreads();
  }
}

template <bool FFT, int KU>
__device__ __forceinline__ void run_batched(const pgx_program& P, const pgx_instance* __restrict__ insts,
                                            const int32_t* __restrict__ work) {
  extern __shared__ __align__(16) double smem_dyn[];
  pgx_instance* sI = reinterpret_cast<pgx_instance*>(smem_dyn);
  const int inst = work[2 * blockIdx.x], tile = work[2 * blockIdx.x + 1];
  const int nwords = sizeof(pgx_instance) / 8;
  const double* src = reinterpret_cast<const double*>(insts + inst);
  double* dst = reinterpret_cast<double*>(sI);
  for (int i = threadIdx.x; i < nwords; i += blockDim.x) dst[i] = src[i];
  __syncthreads();
  run_program<FFT, KU>(P, *sI, tile, smem_dyn + (sizeof(pgx_instance) + 7) / 8);
}

// ------------------------------------------------------------- persistent steps
// Shared memory of a persistent CTA: the current item's descriptor, its program, then the slots.
constexpr int kPersistHead = (int)(((sizeof(pgx_instance) + 15) / 16 + (sizeof(pgx_program) + 15) / 16) * 16);

__device__ __forceinline__ int ld_acquire_gpu(const int32_t* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__global__ void __launch_bounds__(PGX_MAX_THREADS_FFT) line_program_persistent(
    const pgx_program* __restrict__ progs, int nprogs, const pgx_instance* __restrict__ descs, int ndescs,
    const pgx_persist_item* __restrict__ items, int nitems, int32_t* __restrict__ counters, int ncounters,
    int32_t* __restrict__ state, long long spin_limit) {
  extern __shared__ __align__(16) double smem_dyn[];
  pgx_instance* sI = reinterpret_cast<pgx_instance*>(smem_dyn);
  pgx_program* sP = reinterpret_cast<pgx_program*>(reinterpret_cast<char*>(smem_dyn) +
                                                   ((sizeof(pgx_instance) + 15) / 16) * 16);
  double* slots = smem_dyn + kPersistHead / 8;
  __shared__ int s_item, s_go;
  volatile int32_t* err = state + 1;
  // thread 0 holds the index of the CTA's next item: taken from the queue while the current item
  // runs, so the atomic's latency hides behind the tile (items are still taken in list order, and a
  // CTA holds its next item only while it runs one below it: the lowest unfinished item can always run)
  int next = 0;
  if (threadIdx.x == 0) next = atomicAdd(state, 1);
  for (;;) {
    if (threadIdx.x == 0) {
      int it = *err ? nitems : next;
      int go = it < nitems;
      if (go) {
        const pgx_persist_item w = items[it];
        if (w.prog < 0 || w.prog >= nprogs || w.desc < 0 || w.desc >= ndescs || w.done < 0 || w.done >= ncounters ||
            w.wait >= ncounters || w.tile < 0) {
          atomicCAS(state + 1, 0, PGX_PERSIST_BAD_ITEM);
          state[2] = it;
          go = 0;
        } else if (w.wait >= 0) {
          // bounded wait for the items this one depends on (all handed out earlier, to running CTAs)
          const long long t0 = clock64();
          while (ld_acquire_gpu(counters + w.wait) < w.need) {
            if (*err || clock64() - t0 > spin_limit) {
              if (atomicCAS(state + 1, 0, PGX_PERSIST_TIMEOUT) == 0) state[2] = it;
              go = 0;
              break;
            }
            __nanosleep(100);
          }
          __threadfence();  // the producers' results are read with plain loads from here on
        }
        if (go) next = atomicAdd(state, 1);
      }
      s_item = it;
      s_go = go;
    }
    __syncthreads();
    if (!s_go) return;
    const pgx_persist_item w = items[s_item];
    {
      const double* src = reinterpret_cast<const double*>(descs + w.desc);
      double* dst = reinterpret_cast<double*>(sI);
      for (int i = threadIdx.x; i < (int)(sizeof(pgx_instance) / 8); i += blockDim.x) dst[i] = src[i];
      // the program's header and the ops it uses (not all PGX_MAX_OPS)
      const pgx_program* gp = progs + w.prog;
      const int words = (int)((offsetof(pgx_program, ops) + sizeof(pgx_op) * (size_t)min(max(gp->nops, 0),
                                                                                          PGX_MAX_OPS)) / 4);
      const int* ps = reinterpret_cast<const int*>(gp);
      int* pd = reinterpret_cast<int*>(sP);
      for (int i = threadIdx.x; i < words; i += blockDim.x) pd[i] = ps[i];
    }
    __syncthreads();
    run_program<true, 4>(*sP, *sI, w.tile, slots);
    // run_program ends every op with a block barrier: every store of the tile is done here
    if (threadIdx.x == 0) {
      __threadfence();
      atomicAdd(counters + w.done, 1);
    }
  }
}

// Two builds of the interpreter: with the FFT code (programs with DCT ops; up to 768 threads,
// 80 registers a thread without spills) and without it (up to 1024 threads, 64 registers).
__global__ void __launch_bounds__(PGX_MAX_THREADS) line_program_single(const __grid_constant__ pgx_program P,
                                                                       const __grid_constant__ pgx_instance I) {
  extern __shared__ __align__(16) double smem_dyn[];
  run_program<false, 1>(P, I, blockIdx.x, smem_dyn);
}

__global__ void __launch_bounds__(PGX_MAX_THREADS_FFT) line_program_single_fft(const __grid_constant__ pgx_program P,
                                                                               const __grid_constant__ pgx_instance I) {
  extern __shared__ __align__(16) double smem_dyn[];
  run_program<true, 1>(P, I, blockIdx.x, smem_dyn);
}

__global__ void __launch_bounds__(PGX_MAX_THREADS) line_program_batched(const __grid_constant__ pgx_program P,
                                                                        const pgx_instance* __restrict__ insts,
                                                                        const int32_t* __restrict__ work) {
  run_batched<false, 4>(P, insts, work);
}

__global__ void __launch_bounds__(PGX_MAX_THREADS_FFT) line_program_batched_fft(
    const __grid_constant__ pgx_program P, const pgx_instance* __restrict__ insts, const int32_t* __restrict__ work) {
  run_batched<true, 4>(P, insts, work);
}

// The same builds for launches of fewer CTAs than the GPU has SMs (single instances): each CTA's
// ops are one latency chain with nothing to overlap, and the loops that batch several elements'
// loads a thread cost there more than they hide.
__global__ void __launch_bounds__(PGX_MAX_THREADS) line_program_batched_lat(const __grid_constant__ pgx_program P,
                                                                            const pgx_instance* __restrict__ insts,
                                                                            const int32_t* __restrict__ work) {
  run_batched<false, 1>(P, insts, work);
}

__global__ void __launch_bounds__(PGX_MAX_THREADS_FFT) line_program_batched_fft_lat(
    const __grid_constant__ pgx_program P, const pgx_instance* __restrict__ insts, const int32_t* __restrict__ work) {
  run_batched<true, 1>(P, insts, work);
}

}  // namespace pgx

// ---------------------------------------------------------------------------
// Launch helpers used by the C ABI (pgx_api.cu).
extern "C" int64_t pgx_program_smem(const pgx_program* P) {
  int64_t nbuf = P->nslots + 1;
  int64_t doubles = nbuf * P->tb * P->lcap;
  doubles += doubles & 1;
  const int64_t fs = pgx_fft_slots(*P);
  // no FFT buffers (transforms in the slots), or the second one in the spare slot
  const int64_t nbufs = pgx_fft_in_slot(*P) ? 0 : (pgx_fft_in_spare(*P) ? 1 : 2);
  if (P->fft_n > 1) doubles += nbufs * 2 * fs * (int64_t)((P->tb + 1) / 2) * pgx_fft_stride(P->fft_n) + fs * P->tb + 1;
  return doubles * 8;
}

namespace pgx {
// The dynamic shared-memory cap is an attribute of the kernel in the device's
// context, shared by every host thread (the autograd engine launches from its
// own thread): raise it once per device to the opt-in maximum -- it is only a
// cap -- rather than track a per-thread high-water mark that another thread
// could invalidate by setting a lower value.
static int raise_smem_cap_once(const void* fn, int which) {
  static std::mutex mu;
  static bool done[7][64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return (int)e;
  if (dev < 0 || dev >= 64) return (int)cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(mu);
  if (done[which][dev]) return 0;
  int optin = 0;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return (int)e;
  cudaFuncAttributes fa;
  e = cudaFuncGetAttributes(&fa, fn);
  if (e != cudaSuccess) return (int)e;
  // the cap covers dynamic shared memory; the kernel's static shared memory comes on top
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
  if (e != cudaSuccess) return (int)e;
  done[which][dev] = true;
  return 0;
}
static int raise_smem_cap(const void* fn, int which) {
  const int e = raise_smem_cap_once(fn, which);
  if (e) cudaGetLastError();  // a failed call leaves no pending error for the next launch to report
  return e;
}

int launch_single(const pgx_program* P, const pgx_instance* I, cudaStream_t s, int ntiles) {
  int64_t smem = pgx_program_smem(P);
  const bool fft = pgx_has_dct(*P);
  if (smem > 48 * 1024) {
    int e = fft ? raise_smem_cap((const void*)line_program_single_fft, 2)
                : raise_smem_cap((const void*)line_program_single, 0);
    if (e) return e;
  }
  if (fft) line_program_single_fft<<<ntiles, P->nthreads, smem, s>>>(*P, *I);
  else line_program_single<<<ntiles, P->nthreads, smem, s>>>(*P, *I);
  return (int)cudaGetLastError();
}

int persistent_shape(const pgx_program* progs, int nprogs, int threads, int* out_threads, int* ctas_per_sm,
                     int64_t* smem) {
  int64_t need = 0;
  int nt = 32;
  for (int i = 0; i < nprogs; ++i) {
    const int64_t m = pgx_program_smem(progs + i);
    if (m > need) need = m;
    if (progs[i].nthreads > nt) nt = progs[i].nthreads;
  }
  if (threads > 0) nt = threads;
  need += kPersistHead;
  int e = raise_smem_cap((const void*)line_program_persistent, 4);
  if (e) return e;
  int per = 0;
  cudaError_t ce = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, line_program_persistent, nt, (size_t)need);
  if (ce != cudaSuccess) {
    cudaGetLastError();
    return (int)ce;
  }
  *out_threads = nt;
  *ctas_per_sm = per;
  *smem = need;
  return 0;
}

int launch_persistent(const pgx_program* d_progs, int nprogs, const pgx_instance* d_descs, int ndescs,
                      const pgx_persist_item* d_items, int nitems, int32_t* d_counters, int ncounters,
                      int32_t* d_state, int ctas, int threads, int64_t smem, long long spin_limit, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(d_counters, 0, sizeof(int32_t) * (size_t)ncounters, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_state, 0, 3 * sizeof(int32_t), s);
  if (e != cudaSuccess) return (int)e;
  line_program_persistent<<<ctas, threads, smem, s>>>(d_progs, nprogs, d_descs, ndescs, d_items, nitems, d_counters,
                                                      ncounters, d_state, spin_limit);
  return (int)cudaGetLastError();
}

// SMs of the current device, looked up once per device.
static int sm_count() {
  static std::mutex mu;
  static int count[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
  std::lock_guard<std::mutex> lk(mu);
  if (count[dev] == 0 && cudaDeviceGetAttribute(&count[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    count[dev] = 0;
  }
  return count[dev];
}

int launch_batched(const pgx_program* P, const pgx_instance* d_insts, const int32_t* d_work, int nwork,
                   cudaStream_t s) {
  int64_t smem = pgx_program_smem(P) + ((sizeof(pgx_instance) + 15) / 16) * 16;
  const bool fft = pgx_has_dct(*P);
  const bool lat = nwork < sm_count();  // fewer CTAs than SMs: the latency build
  const void* fn = fft ? (lat ? (const void*)line_program_batched_fft_lat : (const void*)line_program_batched_fft)
                       : (lat ? (const void*)line_program_batched_lat : (const void*)line_program_batched);
  if (smem > 48 * 1024) {
    int e = raise_smem_cap(fn, fft ? (lat ? 6 : 3) : (lat ? 5 : 1));
    if (e) return e;
  }
  if (fft) {
    if (lat) line_program_batched_fft_lat<<<nwork, P->nthreads, smem, s>>>(*P, d_insts, d_work);
    else line_program_batched_fft<<<nwork, P->nthreads, smem, s>>>(*P, d_insts, d_work);
  } else {
    if (lat) line_program_batched_lat<<<nwork, P->nthreads, smem, s>>>(*P, d_insts, d_work);
    else line_program_batched<<<nwork, P->nthreads, smem, s>>>(*P, d_insts, d_work);
  }
  return (int)cudaGetLastError();
}
}  // namespace pgx
