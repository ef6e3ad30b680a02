// Device kernels of the GB300 ILU0-BiCGSTAB path (sm_103a).
//
// Every kernel is memory-streaming work on the sliced layout described in
// gbilu_host.hpp: one thread owns one block row (3 unknowns), a warp owns a
// 32-row slice, and each of the 9 block entries of a slot is one coalesced
// 32-lane load. Dot products and norms are fused into the kernel that
// produces the vector; per-CTA partials are combined by the last CTA to
// finish ("last block" pattern, no spinning), in a fixed order, so every
// result is bit-for-bit reproducible from run to run.
//
// Solver scalars never leave the device: they live in a Ctl block that the
// fused kernels update; every kernel of an iteration returns at once when
// Ctl::done is set, which lets a fixed CUDA graph run the loop.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace gbilu {

constexpr int kThreads = 256;                 // threads per CTA
constexpr int kWarps = kThreads / 32;
constexpr double kAlreadySolved = 1e-30;      // constants.vhd:59

enum Status {
  ST_OK = 0, ST_MAXIT = 1, ST_ALREADY = 2, ST_BREAKDOWN = 3, ST_NONFINITE = 4,
  ST_TIMEOUT = 5
};

constexpr int kMaxPhases = 96;                // color steps of one ILU apply

// Device-resident solver state, one per solve in flight.
struct Ctl {
  double rho, alpha, omega, beta;
  double bound, norm0, norm, tol;
  double norms[4];
  double dots[4];                 // last reduced values (diagnostics)
  int absolute, maxit;
  int last_norm_idx;
  int half;                       // the reference's half-iteration counter
  int k;                          // current full iteration
  int done, status, stop_half;    // stop_half: stopped after a first half
  unsigned long long t_start, timeout_ns;
  unsigned int counter[8];        // arrival counters of the last-block pattern
  unsigned int bar_count, bar_gen;  // grid barrier of cooperative launches
  int bar_fail;                   // a barrier wait timed out
  int body_runs;                  // loop bodies run (graph launches count)
  // mixed precision by residual replacement (reliable updates): the FP32
  // iteration works on (quantity / sigma); x and the true residual are FP64
  int ru_mode;                    // 1: stops are decided on the true residual
  int ru;                         // a replacement is due at the end of this iteration
  double sigma;                   // scale of the FP32 vectors (the initial ||r||)
  double ru_delta;                // replace when ||r|| < ru_delta * rmax
  double rmax;                    // largest recursive ||r|| since the last replacement
  double rho_prev;                // rho before the last update_r (for beta after a replacement)
  double true_norm;               // ||b - A x|| of the last replacement (FP64)
  int replacements;
  unsigned long long phase_ns[kMaxPhases + 1];   // traced ILU apply: phase starts
  unsigned int step_next[kMaxPhases];   // single-launch apply: next slice of a large step
};

// --------------------------------------------------------------------------
// small helpers
// --------------------------------------------------------------------------

template <typename T> __device__ __forceinline__ T ldg_stream(const T *p) { return __ldcs(p); }

// Entry e (row-major in the 3x3 block) of lane l in slot `slot` of a sliced
// value array of V; the D^-1 arrays use the same layout with one slot per
// slice. FP64: [(slot*9 + e)*32 + l], entry-major, each of a warp's 9 loads
// one coalesced 256-byte access. FP32: the slot's 288 values in three groups,
// entries 0-3 and 4-7 with their 4 floats consecutive per lane and entry 8
// with one float per lane, so that a lane reads its block with two 16-byte
// loads and one 4-byte load instead of nine (each warp load still one
// contiguous range): the FP32 SpMV and sweeps wait less on the load queue.
template <typename V> __host__ __device__ inline size_t sl_idx(size_t slot, int e, int l) {
  if (sizeof(V) == 4)
    return slot * 288 + (e < 8 ? (size_t)(e >> 2) * 128 + (size_t)l * 4 + (size_t)(e & 3)
                               : 256 + (size_t)l);
  return (slot * 9 + (size_t)e) * 32 + (size_t)l;
}

// The 9 entries of lane l's block in the slot that starts at b, from global
// memory (streaming loads) or from shared memory.
template <typename V, bool GLOBAL>
__device__ __forceinline__ void load_block(const V *b, int l, V (&e)[9]) {
  if constexpr (sizeof(V) == 4) {
    const float4 *q = reinterpret_cast<const float4 *>(b);
    const float4 u = GLOBAL ? __ldcs(q + l) : q[l];
    const float4 w = GLOBAL ? __ldcs(q + 32 + l) : q[32 + l];
    e[0] = u.x; e[1] = u.y; e[2] = u.z; e[3] = u.w;
    e[4] = w.x; e[5] = w.y; e[6] = w.z; e[7] = w.w;
    e[8] = GLOBAL ? __ldcs(b + 256 + l) : b[256 + l];
  } else {
#pragma unroll
    for (int k = 0; k < 9; ++k) e[k] = GLOBAL ? __ldcs(b + k * 32 + l) : b[k * 32 + l];
  }
}

// L2 prefetch of matrix slices ahead of the warp that will read them (the
// large steps of the single-launch apply, the SpMV): rounds of the grid's
// warps ahead; 0 turns it off.
#ifndef GBILU_SPMV_PREFETCH
#define GBILU_SPMV_PREFETCH 0
#endif
#ifndef GBILU_PREFETCH_EVICT_FIRST
#define GBILU_PREFETCH_EVICT_FIRST 1
#endif
// The prefetched lines are marked evict-first, like the streaming loads
// that read them: they must not push the solver's vectors out of L2.
__device__ __forceinline__ void prefetch_l2(const void *p, unsigned int bytes) {
  if (GBILU_PREFETCH_EVICT_FIRST) {
    unsigned long long pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    asm volatile("cp.async.bulk.prefetch.L2.global.L2::cache_hint [%0], %1, %2;" ::"l"(p),
                 "r"(bytes), "l"(pol)
                 : "memory");
  } else {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
  }
}
// The slice's blocks (values and column indices: contiguous, 16-byte
// aligned ranges of the sliced layout) and, when the step reads it, its D
// block; o = off[s], w = off[s + 1] - o.
template <typename V>
__device__ __forceinline__ void prefetch_slice(int s, int o, int w, const int *col, const V *val,
                                               const V *dmat, bool d) {
  if (w > 0) {
    prefetch_l2(val + (size_t)o * 9 * 32, (unsigned int)w * 9 * 32 * (unsigned int)sizeof(V));
    prefetch_l2(col + (size_t)o * 32, (unsigned int)w * 32 * (unsigned int)sizeof(int));
  }
  if (d) prefetch_l2(dmat + (size_t)s * 9 * 32, 9 * 32 * (unsigned int)sizeof(V));
}

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool finite(double v) { return isfinite(v); }

// Exact product and error-free sum on the FP32 pipe: a double-float
// accumulator (hi + lo) that keeps ~44 bits, so FP32 vectors get dot products
// of FP64 quality without touching GB300's slow FP64 units per element.
struct DF {
  float hi, lo;
};
__device__ __forceinline__ void df_add_prod(DF &acc, float a, float b) {
  const float p = a * b;
  const float e = fmaf(a, b, -p);             // a*b = p + e exactly
  const float s = acc.hi + p;
  const float bb = s - acc.hi;
  const float err = (acc.hi - (s - bb)) + (p - bb);
  acc.hi = s;
  acc.lo += err + e;
}
__device__ __forceinline__ double df_value(const DF &a) { return (double)a.hi + (double)a.lo; }

// Deterministic block reduction of NV doubles over a kThreads-thread CTA;
// result valid in thread 0. GB300's FP64 pipe is 1/64 of FP32, so a shuffle
// tree in every warp (45 FP64 warp instructions per CTA) costs microseconds:
// the values go through shared memory instead and warp 0 alone sums them, 8
// per lane in order and then a 5-level shuffle tree (12 instructions).
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV]) {
  __shared__ double red[NV][kThreads];
#pragma unroll
  for (int j = 0; j < NV; ++j) red[j][threadIdx.x] = v[j];
  __syncthreads();
  if (threadIdx.x < 32) {
    const int l = threadIdx.x;
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      double x = red[j][l];
#pragma unroll
      for (int k = 1; k < kWarps; ++k) x += red[j][l + 32 * k];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      v[j] = x;
    }
  }
  __syncthreads();
}

// Writes this CTA's partials and returns true in every thread of the CTA
// that arrives last; that CTA then holds the fixed-order grid totals in tot.
template <int NV>
__device__ __forceinline__ bool grid_sum(double (&v)[NV], double *partials,
                                         unsigned int *counter, double (&tot)[NV]) {
  __shared__ bool last;
  __shared__ double res[NV];
  block_sum<NV>(v);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < NV; ++j) partials[(size_t)j * gridDim.x + blockIdx.x] = v[j];
    // acquire-release arrival: releases this thread's partials and, in the
    // last CTA, acquires everyone's (the CTA barrier below passes that on to
    // its other threads); no separate fences
    unsigned int prev;
    asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], 1;" : "=r"(prev) : "l"(counter) : "memory");
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  double acc[NV];
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    acc[j] = 0.0;
    for (unsigned int b = threadIdx.x; b < gridDim.x; b += blockDim.x)
      acc[j] += __ldcg(partials + (size_t)j * gridDim.x + b);
  }
  block_sum<NV>(acc);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < NV; ++j) res[j] = acc[j];
    *counter = 0u;                               // ready for the next kernel
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < NV; ++j) tot[j] = res[j];
  return true;
}

// the m-th norm after the initial one goes to ring slot (half % 3) + 1
// (solver.vhd:913-918, bicgstab_utils.cpp:256)
__device__ __forceinline__ void push_norm(Ctl *c, double nrm) {
  const int idx = (c->half % 3) + 1;
  c->norms[idx] = nrm;
  c->last_norm_idx = idx;
  c->norm = nrm;
}

__device__ __forceinline__ void stop(Ctl *c, int status, int stop_half) {
  c->status = status;
  c->stop_half = stop_half;
  c->done = 1;
}

// --------------------------------------------------------------------------
// control
// --------------------------------------------------------------------------

__global__ void k_ctl_init(Ctl *c, double tol, int absolute, int maxit,
                           unsigned long long timeout_ns) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    c->rho = c->alpha = c->omega = c->beta = 0.0;
    c->bound = c->norm0 = c->norm = 0.0;
    c->tol = tol;
    for (int i = 0; i < 4; ++i) { c->norms[i] = 0.0; c->dots[i] = 0.0; }
    c->absolute = absolute;
    c->maxit = maxit;
    c->last_norm_idx = 0;
    c->half = -1;
    c->k = 0;
    c->done = 0;
    c->status = ST_MAXIT;
    c->stop_half = 0;
    c->t_start = globaltimer();
    c->timeout_ns = timeout_ns;
    for (int i = 0; i < 8; ++i) c->counter[i] = 0u;
    c->bar_count = 0u;
    c->bar_gen = 0u;
    c->bar_fail = 0;
    c->body_runs = 0;
    c->ru_mode = 0;
    c->ru = 0;
    c->sigma = 1.0;
    c->ru_delta = 0.1;
    c->rmax = 0.0;
    c->rho_prev = 0.0;
    c->true_norm = 0.0;
    c->replacements = 0;
    for (int q = 0; q < kMaxPhases; ++q) c->step_next[q] = 0u;
  }
}

// Solver scalars for timing the iteration's kernels one at a time: unit
// rho, alpha, omega, beta, a zero bound and no iteration limit, so that no
// kernel stops the run.
__global__ void k_ctl_bench(Ctl *c) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    c->rho = c->alpha = c->omega = c->beta = 1.0;
    c->bound = 0.0;
    c->maxit = 0x7fffffff;
    c->half = 0;
    c->k = 0;
    c->done = 0;
    c->ru_mode = 0;
  }
}

// Steps 0/1 of the PROGRAM (solver_pkg.vhd:122-123, solver.vhd:887-911):
// r = b - A x0, rho = ||r||^2, the "already solved" test and the absolute
// stopping bound. MODE 0: r = b - A x (vals/x given); MODE 1: r = b (x0 = 0,
// used by the inner solves of iterative refinement).
template <typename T>
__device__ __forceinline__ void finish_init(Ctl *c, double rr) {
  const double n0 = sqrt(rr);
  c->norm0 = n0;
  c->norm = n0;
  c->norms[0] = n0;
  c->last_norm_idx = 0;
  c->rho = rr;
  double bound = c->absolute ? c->tol : kAlreadySolved;
  if (!finite(n0)) { stop(c, ST_NONFINITE, 0); return; }
  if (!(n0 > bound)) { stop(c, ST_ALREADY, 0); return; }
  if (!c->absolute) bound = c->tol * n0;
  c->bound = bound;
  c->half = 0;
  c->k = 0;
}

// --------------------------------------------------------------------------
// one sliced row: a += sign * sum_k B_k x_{c_k}
// --------------------------------------------------------------------------

#ifndef GBILU_BATCH
#define GBILU_BATCH 4
#endif
constexpr int kBatch = GBILU_BATCH;   // blocks whose loads are in flight together
#ifndef GBILU_BATCH64
#define GBILU_BATCH64 2
#endif
constexpr int kBatch64 = GBILU_BATCH64;   // the same for FP64 values

// Vector loads: CG = through L2 only (ld.global.cg), else through L1. The
// per-SM L1 is not coherent inside one launch; loads of values that other
// SMs may still be writing go through L2 (the small steps poll with relaxed
// gpu-scope loads instead).
template <bool CG, typename T> __device__ __forceinline__ T ldv(const T *p) {
  if (CG) return __ldcg(p);
  return *p;
}

// Column indices are fetched kBatch at a time, so the gathers and the 9
// coalesced value loads of kBatch blocks are in flight together: a row of
// w blocks costs about 2*ceil(w/kBatch) memory round trips instead of 2*w.
// Padding slots (column -1) only occur after a row's last block.
// Neighbour columns below lo are read from xlo instead of x (the first sweep
// reads the input vector for color 0, whose L rows are empty). EARLY: the
// block values are loaded without waiting for the column indices.
template <typename V, typename T, bool NEG, bool CG, bool EARLY>
__device__ __forceinline__ void row_blocks(const int *__restrict__ col, const V *__restrict__ val,
                                           int o, int wdt, int lane, const T *x, const T *xlo,
                                           int lo, T &a0, T &a1, T &a2) {
  // FP64 batches of 2 keep the kernels within 128 registers (the FP64 pipe,
  // not the load latency, bounds them); FP32 batches of kBatch
  constexpr int B = sizeof(V) == 8 ? kBatch64 : kBatch;
  for (int k0 = 0; k0 < wdt; k0 += B) {
    int c[B];
#pragma unroll
    for (int j = 0; j < B; ++j)
      c[j] = (k0 + j < wdt) ? ldg_stream(col + (size_t)(o + k0 + j) * 32 + lane) : -1;
    // all loads of the batch first ... The values of every slot of the
    // slice exist for all 32 lanes (padding: zeros, column -1), so with
    // EARLY they are loaded whatever the column index says and go out
    // together with the index loads instead of after them; only the
    // gathers wait for the index.
    T xv[B][3];
    V b[B][9];
#pragma unroll
    for (int j = 0; j < B; ++j) {
      const V *v = val + (size_t)(o + k0 + j) * 9 * 32;   // the slot
      if (EARLY && k0 + j < wdt) load_block<V, true>(v, lane, b[j]);
      if (c[j] >= 0) {
        const T *xs = c[j] < lo ? xlo : x;
#pragma unroll
        for (int e = 0; e < 3; ++e) xv[j][e] = ldv<CG>(xs + 3 * c[j] + e);
        if (!EARLY) load_block<V, true>(v, lane, b[j]);
      }
    }
    // ... then the multiply-adds
#pragma unroll
    for (int j = 0; j < B; ++j) {
      if (c[j] >= 0) {
        T bb[9];
#pragma unroll
        for (int e = 0; e < 9; ++e) bb[e] = NEG ? -(T)b[j][e] : (T)b[j][e];
        a0 = fma(bb[0], xv[j][0], a0); a0 = fma(bb[1], xv[j][1], a0); a0 = fma(bb[2], xv[j][2], a0);
        a1 = fma(bb[3], xv[j][0], a1); a1 = fma(bb[4], xv[j][1], a1); a1 = fma(bb[5], xv[j][2], a1);
        a2 = fma(bb[6], xv[j][0], a2); a2 = fma(bb[7], xv[j][1], a2); a2 = fma(bb[8], xv[j][2], a2);
      }
    }
    if (c[B - 1] < 0) break;
  }
}

// --------------------------------------------------------------------------
// sliced SpMV with fused reductions
// --------------------------------------------------------------------------

enum SpmvMode { SPMV_PLAIN = 0, SPMV_RESID = 1, SPMV_ALPHA = 2, SPMV_OMEGA = 3, SPMV_TRUE = 4 };

// y = A x over all slices. RESID: y = b - A x, ||y||^2 -> init. ALPHA:
// (y, w) -> alpha = rho/(y,w) (step 5). OMEGA: (y, w), (y, y) ->
// omega = (y,w)/(y,y) (step 10). TRUE: y = b - A x and ||y|| into
// Ctl::true_norm, only when a residual replacement is due.
// V: matrix value type, T: vector type.
// CTAs per SM the register budget must allow: three in both precisions
// (80 registers, no spills). The FP32 SpMV is HBM-bound and gains from the
// third CTA; in FP64 the plain mode fits three anyway, and the modes with
// fused dots (88-90 registers with two) gain 2.5 % per solve iteration.
#ifndef GBILU_SPMV32_MINB
#define GBILU_SPMV32_MINB 3
#endif
#ifndef GBILU_SPMV64_MINB
#define GBILU_SPMV64_MINB 3
#endif
// x_nonzero (PLAIN only, may be null): a flag the producer of x set when
// any entry of x is not zero; when it is clear y = A x = 0 is written
// without reading A (the initial residual of a solve from x0 = 0).
template <typename V, typename T, int MODE>
__global__ void __launch_bounds__(kThreads, sizeof(V) == 4 ? GBILU_SPMV32_MINB : GBILU_SPMV64_MINB)
k_spmv(Ctl *ctl, int S, const int2 *__restrict__ srows, const int *__restrict__ off,
       const int *__restrict__ col, const V *__restrict__ val, const T *__restrict__ x,
       T *__restrict__ y, const T *__restrict__ w, double *partials,
       const int *x_nonzero = nullptr) {
  if (MODE == SPMV_TRUE && (!ctl->ru || ctl->done)) return;
  if (MODE != SPMV_PLAIN && MODE != SPMV_RESID && ctl->done) return;
  if (MODE == SPMV_PLAIN && x_nonzero && !*x_nonzero) {
    const int n = 3 * (srows[S - 1].x + srows[S - 1].y);
    for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads)
      y[i] = (T)0;
    return;
  }
  constexpr bool RES = MODE == SPMV_RESID || MODE == SPMV_TRUE;
  // persistent grid: each warp walks slices warp, warp + all warps, ...;
  // one reduction per CTA at the end instead of one per 8 slices
  const int lane = threadIdx.x & 31;
  const int nwarps = gridDim.x * kWarps;
  double d1 = 0.0, d2 = 0.0;
  DF f1 = {0.f, 0.f}, f2 = {0.f, 0.f};
  // FP32: the next slice's row range and slot range are loaded while this
  // one is computed (one dependent round trip less per slice; the mixed
  // solve gains 1.5 %). FP64 is bound by the FP64 unit, and the extra
  // registers spill in its dot modes: it loads them per slice.
  constexpr bool AHEAD = sizeof(V) == 4;
  // values loaded ahead of the column indices in FP32; the FP64 SpMV with
  // fused dots ran 1-3 % slower that way (FP64 unit bound)
  constexpr bool kSpmvEarly = sizeof(V) == 4;
#if GBILU_SPMV_PREFETCH > 0
  // FP32 matrices only: the FP64 SpMV is bound by the FP64 unit
  constexpr bool PF = sizeof(V) == 4;
#endif
  int s = blockIdx.x * kWarps + (threadIdx.x >> 5);
  int2 sr_n = make_int2(0, 0);
  int o_n = 0, e_n = 0;
  if (AHEAD && s < S) { sr_n = srows[s]; o_n = off[s]; e_n = off[s + 1]; }
#if GBILU_SPMV_PREFETCH > 0
  // the first rounds of this warp's slices asked from L2 here (lane k:
  // round k), then the slice GBILU_SPMV_PREFETCH rounds ahead of each
  if (PF && lane < GBILU_SPMV_PREFETCH && s + lane * nwarps < S) {
    const int sp = s + lane * nwarps, po = off[sp];
    prefetch_slice<V>(sp, po, off[sp + 1] - po, col, val, val, false);
  }
#endif
  for (; s < S; s += nwarps) {
#if GBILU_SPMV_PREFETCH > 0
    const int sp = s + GBILU_SPMV_PREFETCH * nwarps;
    const int po = PF && lane == 0 && sp < S ? off[sp] : 0;
    const int pe = PF && lane == 0 && sp < S ? off[sp + 1] : 0;
#endif
    int2 sr;
    int o, wdt;
    if (AHEAD) {
      sr = sr_n; o = o_n; wdt = e_n - o_n;
      if (s + nwarps < S) {
        sr_n = srows[s + nwarps]; o_n = off[s + nwarps]; e_n = off[s + nwarps + 1];
      }
    } else {
      sr = srows[s]; o = off[s]; wdt = off[s + 1] - o;
    }
    if (lane < sr.y) {
      const int row = sr.x + lane;
      T a0 = 0, a1 = 0, a2 = 0;
      row_blocks<V, T, false, false, kSpmvEarly>(col, val, o, wdt, lane, x, x, 0, a0, a1, a2);
      if (RES) {
        a0 = w[3 * row] - a0; a1 = w[3 * row + 1] - a1; a2 = w[3 * row + 2] - a2;
      }
      y[3 * row] = a0; y[3 * row + 1] = a1; y[3 * row + 2] = a2;
      if (RES) {
        if (sizeof(T) == 8) d1 += (double)a0 * a0 + (double)a1 * a1 + (double)a2 * a2;
        else { df_add_prod(f1, (float)a0, (float)a0); df_add_prod(f1, (float)a1, (float)a1); df_add_prod(f1, (float)a2, (float)a2); }
      } else if (MODE == SPMV_ALPHA || MODE == SPMV_OMEGA) {
        const T w0 = w[3 * row], w1 = w[3 * row + 1], w2 = w[3 * row + 2];
        if (sizeof(T) == 8) {
          d1 += (double)a0 * w0 + (double)a1 * w1 + (double)a2 * w2;
          if (MODE == SPMV_OMEGA) d2 += (double)a0 * a0 + (double)a1 * a1 + (double)a2 * a2;
        } else {
          df_add_prod(f1, (float)a0, (float)w0); df_add_prod(f1, (float)a1, (float)w1); df_add_prod(f1, (float)a2, (float)w2);
          if (MODE == SPMV_OMEGA) { df_add_prod(f2, (float)a0, (float)a0); df_add_prod(f2, (float)a1, (float)a1); df_add_prod(f2, (float)a2, (float)a2); }
        }
      }
    }
#if GBILU_SPMV_PREFETCH > 0
    if (PF && lane == 0 && sp < S) prefetch_slice<V>(sp, po, pe - po, col, val, val, false);
#endif
  }
  if (MODE == SPMV_PLAIN) return;
  if (sizeof(T) == 4) { d1 = df_value(f1); d2 = df_value(f2); }
  if (MODE == SPMV_RESID) {
    double v[1] = {d1}, tot[1];
    if (grid_sum<1>(v, partials, &ctl->counter[0], tot) && threadIdx.x == 0)
      finish_init<T>(ctl, tot[0]);
  } else if (MODE == SPMV_TRUE) {
    double v[1] = {d1}, tot[1];
    if (grid_sum<1>(v, partials, &ctl->counter[0], tot) && threadIdx.x == 0)
      ctl->true_norm = sqrt(tot[0]);
  } else if (MODE == SPMV_ALPHA) {
    double v[1] = {d1}, tot[1];
    if (grid_sum<1>(v, partials, &ctl->counter[1], tot) && threadIdx.x == 0) {
      const double a = ctl->rho / tot[0];
      ctl->dots[0] = tot[0];
      ctl->alpha = a;
      if (tot[0] == 0.0 || !finite(a)) stop(ctl, ST_BREAKDOWN, 0);
    }
  } else {
    double v[2] = {d1, d2}, tot[2];
    if (grid_sum<2>(v, partials, &ctl->counter[2], tot) && threadIdx.x == 0) {
      const double om = tot[0] / tot[1];
      ctl->dots[1] = tot[0];
      ctl->dots[2] = tot[1];
      ctl->omega = om;
      // half 1 already advanced x by alpha p^: keep it on a stop here
      if (tot[1] == 0.0 || !finite(om)) stop(ctl, ST_BREAKDOWN, 1);
    }
  }
}

// --------------------------------------------------------------------------
// one color of a triangular sweep
// --------------------------------------------------------------------------

// One color step of a preconditioner apply: rows [row0, row0 + nrows)
// starting at slice slice0 of matrix mat (0: L, or U^T in the adjoint; 1: U,
// or L^T). The first sweep (L forward; U^T in the adjoint) writes its result
// y to ybuf for every row of the color, and for the rows from final0 on --
// those with no neighbour of a higher color, ordered last in their color --
// the final value hat = [D] y right away. The second sweep (U backward; L^T)
// then only covers the leading rows of each color: hat = [D] (ybuf - B hat).
// Color 0 has no L rows: its y is the input itself (src).
// L sweep: ilu0.vhd:413-416, colors ascending (sparstition.vhd:751-756);
// U sweep with D^-1: ilu0.vhd:293-323,407-411, colors descending.
struct Phase {
  int row0, nrows, slice0, mat;
  int has_d;      // D applied to the row result (the adjoint's U^T step: D^-T)
  int own_y;      // own rows read ybuf (second sweep) instead of src
  int nbr_hat;    // neighbours read hat (second sweep) instead of ybuf
  int src_rows;   // first sweep: neighbour rows below this read src (color 0)
  int to_y;       // first sweep: the result goes to ybuf ...
  int final0;     // ... and rows from final0 on are final: hat = [D] result
  int final_d;    //     with D = D^-1 (forward) or the identity (adjoint)
  int staged;     // the step's matrix rows come from shared memory
  int local_after;  // this step and the next have one slice each and run on
                    // CTA 0: a CTA barrier between them instead of a grid one
  int flow_after;   // this step and the next are small: when both are staged,
                    // no barrier -- the next step waits for the values it reads
  int streamed;     // a large step whose slices a producer warp streams into
                    // a shared-memory ring ahead of the compute warps
  // whether a D block of the step's rows is read
  __host__ __device__ bool uses_d() const { return has_d || (to_y && final_d); }
};

// d0 a0 + d1 a1 + d2 a2 in one fixed operation order (every path that
// applies a D block uses it, so they agree bit for bit)
template <typename T>
__device__ __forceinline__ T dot3(T d0, T d1, T d2, T a0, T a1, T a2) {
  return fma(d2, a2, fma(d1, a1, d0 * a0));
}

// (a0, a1, a2) <- D (a0, a1, a2) with D lane l's block of the slot at d
template <typename V, typename T, bool GLOBAL>
__device__ __forceinline__ void apply_dp(const V *d, int l, T &a0, T &a1, T &a2) {
  V dv[9];
  load_block<V, GLOBAL>(d, l, dv);
  T dd[9];
#pragma unroll
  for (int e = 0; e < 9; ++e) dd[e] = (T)dv[e];
  const T z0 = dot3(dd[0], dd[1], dd[2], a0, a1, a2);
  const T z1 = dot3(dd[3], dd[4], dd[5], a0, a1, a2);
  const T z2 = dot3(dd[6], dd[7], dd[8], a0, a1, a2);
  a0 = z0; a1 = z1; a2 = z2;
}

// Stores one row's result as the phase says (d: the slot of the row's D
// block, l: the row's lane).
template <typename V, typename T, bool GLOBAL>
__device__ __forceinline__ void phase_store(const Phase &P, int row, const V *d, int l, T a0,
                                            T a1, T a2, T *ybuf, T *hat) {
  if (P.has_d) apply_dp<V, T, GLOBAL>(d, l, a0, a1, a2);
  if (P.to_y) {
    ybuf[3 * row] = a0; ybuf[3 * row + 1] = a1; ybuf[3 * row + 2] = a2;
    if (row < P.final0) return;
    if (P.final_d) apply_dp<V, T, GLOBAL>(d, l, a0, a1, a2);
  }
  hat[3 * row] = a0; hat[3 * row + 1] = a1; hat[3 * row + 2] = a2;
}

#ifndef GBILU_D_PREFETCH
#define GBILU_D_PREFETCH 1
#endif
// One row of a step, one thread: a = own_i - sum_j B_ij nbr_j, then stored.
template <typename V, typename T, bool CG>
__device__ __forceinline__ void phase_row(const Phase &P, int row, int s, int lane,
                                          const int *__restrict__ off, const int *__restrict__ col,
                                          const V *__restrict__ val, const V *__restrict__ dmat,
                                          const T *src, T *ybuf, T *hat) {
  const T *own = P.own_y ? ybuf : src;
  if (GBILU_D_PREFETCH && (P.has_d || (P.to_y && P.final_d && row - lane + 31 >= P.final0))) {
    // the slice's D block (9 * 32 values, one 128-byte line per lane) is
    // read at the end of the row: asked from L2 now, without registers
    constexpr int kLines = 9 * 32 * (int)sizeof(V) / 128;
    if (lane < kLines)
      asm volatile("prefetch.global.L2 [%0];" ::"l"(dmat + (size_t)s * 9 * 32 +
                                                     lane * (128 / (int)sizeof(V))));
  }
  const int o = off[s], wdt = off[s + 1] - o;
  T a0 = ldv<CG>(own + 3 * row), a1 = ldv<CG>(own + 3 * row + 1), a2 = ldv<CG>(own + 3 * row + 2);
  row_blocks<V, T, true, CG, true>(col, val, o, wdt, lane, P.nbr_hat ? hat : ybuf, src, P.src_rows, a0,
                             a1, a2);
  phase_store<V, T, true>(P, row, dmat + (size_t)s * 9 * 32, lane, a0, a1, a2, ybuf, hat);
}

// Colors with at most kSmallRows rows cannot fill the GPU: their steps are
// latency-bound and the single-launch apply stages them in shared memory.
constexpr int kSmallRows = 16384;

// One step per launch (the per-color mode; the same row arithmetic as the
// single-launch apply, so both give identical bits).
template <typename V, typename T>
__global__ void __launch_bounds__(kThreads, 2)
k_phase(const Ctl *ctl, Phase P, const int *__restrict__ off, const int *__restrict__ col,
        const V *__restrict__ val, const V *__restrict__ dmat, const T *src, T *ybuf, T *hat) {
  if (ctl->done) return;
  const int t = blockIdx.x * kThreads + threadIdx.x;
  if (t >= P.nrows) return;
  phase_row<V, T, false>(P, P.row0 + t, P.slice0 + (t >> 5), t & 31, off, col, val, dmat, src,
                         ybuf, hat);
}

// --------------------------------------------------------------------------
// whole preconditioner apply in one cooperative launch
// --------------------------------------------------------------------------

struct PhaseList {
  int n;
  int trace;                      // CTA 0 stamps %globaltimer at each phase start
  Phase p[kMaxPhases];
};

// Small color steps are latency-bound: their slices (values, column
// indices, inverse diagonal blocks) are copied into shared memory with TMA
// bulk copies when the launch starts, so that the step itself only gathers
// the neighbour values from L2. The host assigns slices to CTAs; entry
// e of CTA b says: phase q, slice j of that phase's color, row width w, and
// the byte offset pos of [values | column indices | D^-1] in shared memory.
struct StageEntry {
  int q, j, w, pos;
};
constexpr int kMaxStage = 64;         // entries per CTA

// Large color steps stream their slices through a ring of ring_ns stages
// of ring_stride bytes at byte offset ring_off of the dynamic shared memory
// (after the staged small steps): the producer warp copies a slice's
// [values | column indices | D block] with bulk copies as soon as its stage
// is free -- running ahead into the next large step while the small steps
// and barriers in between run -- and the compute warps take the slices in
// turn. ring_ns = 0: no ring, every warp computes and the large steps load
// their matrix rows directly.
constexpr int kRingMax = 16;

struct StagePlan {
  const StageEntry *tab;              // [grid][kMaxStage]
  const int2 *cnt;                    // per CTA: entries, total bytes
  int enabled;
  int ring_ns, ring_stride, ring_off;
  // per CTA, its streamed slices in launch order: entry g of CTA b at
  // ring_tab[b * ring_max + g] = slice | matrix << 30 | uses_d << 31
  // (matrix 1: the second sweep's), ring_cnt[b] of them
  const unsigned int *ring_tab;
  const int *ring_cnt;
  int ring_max;
};

constexpr unsigned int kStageSpins = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// non-blocking phase test (try_wait may suspend the thread for a while,
// which in a divergent warp holds up the other lanes)
__device__ __forceinline__ bool mbar_test_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// global -> shared bulk copy (16-byte aligned ends, size a multiple of 16),
// completion counted on the mbarrier
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

#ifndef GBILU_COOP_THREADS
#define GBILU_COOP_THREADS 512
#endif
constexpr int kCoopThreads = GBILU_COOP_THREADS;   // one CTA per SM: half the barrier arrivals
// threads per CTA of the single-launch apply by vector precision
#ifndef GBILU_COOP_THREADS64
#define GBILU_COOP_THREADS64 GBILU_COOP_THREADS
#endif
#ifndef GBILU_COOP_THREADS32
#define GBILU_COOP_THREADS32 GBILU_COOP_THREADS
#endif
template <typename T> __host__ __device__ constexpr int coop_threads() {
  return sizeof(T) == 4 ? GBILU_COOP_THREADS32 : GBILU_COOP_THREADS64;
}

// Every spin is bounded: a barrier that does not complete within this many
// polls marks the run failed (Ctl::bar_fail) and the kernel returns.
constexpr unsigned int kBarrierSpins = 1u << 22;

__device__ __forceinline__ unsigned int atom_add_release(unsigned int *p, unsigned int v) {
  unsigned int old;
  asm volatile("atom.add.release.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ unsigned int ld_acquire(const unsigned int *p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Ticket grid barrier for a cooperative launch (all CTAs resident). The
// counter only grows: every CTA adds 1 per barrier with release semantics
// (after bar.sync, so it publishes the whole CTA's writes) and waits with
// acquire loads until the counter reaches the end of its round. It starts at
// 0 per solve (k_ctl_init) and every launch that uses it has the same grid
// size, so rounds never straddle launches. One atomic and one poll per CTA
// instead of fence + atomic + fence + atomic. Returns false after a timed-out
// wait.
// late: this thread's own wait before the barrier ran out; if any thread of
// the CTA says so, the CTA still takes part in the barrier (the others do
// not wait for it in vain), marks the run failed and gets false.
__device__ __forceinline__ void mark_stage_timeout(Ctl *c) {
  atomicExch(&c->bar_fail, 2);
  c->status = ST_TIMEOUT;
  __threadfence();
  atomicExch(&c->done, 1);
}

// CTA barriers over the first nthreads threads (named barrier 7): the
// compute warps of the single-launch apply, which leaves its producer warp
// out of them once the two roles split.
__device__ __forceinline__ void cta_sync(int nthreads) {
  asm volatile("bar.sync 7, %0;" ::"r"(nthreads) : "memory");
}
__device__ __forceinline__ int cta_sync_or(int nthreads, int pred) {
  int r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.s32 p, %1, 0;\n bar.red.or.pred q, 7, %2, p;\n"
      " selp.s32 %0, 1, 0, q;\n}\n"
      : "=r"(r)
      : "r"(pred), "r"(nthreads)
      : "memory");
  return r;
}

__device__ __forceinline__ bool grid_barrier(Ctl *c, bool late = false, int nthreads = 0) {
  __shared__ int ok;
  if (nthreads == 0) nthreads = blockDim.x;
  const int any_late = cta_sync_or(nthreads, late);
  if (threadIdx.x == 0) {
    ok = !any_late;
    if (any_late) mark_stage_timeout(c);
    __threadfence();   // the CTA's writes (ordered by bar.sync) before the ticket
    const unsigned int ticket = atom_add_release(&c->bar_count, 1u);
    const unsigned int target = (ticket / gridDim.x + 1) * gridDim.x;
    unsigned int spins = 0;
    while ((int)(ld_acquire(&c->bar_count) - target) < 0) {
      if (++spins > kBarrierSpins) {
        ok = 0;
        atomicExch(&c->bar_fail, 1);
        c->status = ST_TIMEOUT;     // the solve stops: every later kernel
        __threadfence();            // of the run sees done and returns
        atomicExch(&c->done, 1);
        break;
      }
      if (spins > 256) __nanosleep(32);
    }
  }
  cta_sync(nthreads);
  return ok != 0;
}

// Runs of consecutive staged steps are ordered by the data instead of grid
// barriers: when the launch starts, every CTA sets the outputs (y and z
// rows) of its staged rows to a sentinel, a NaN payload that arithmetic
// never produces (its NaNs are canonical, and every staged output is an
// arithmetic result), and a consumer that loads a sentinel loads again
// until the producer's value is there. One memory round trip per dependency
// instead of a barrier's fence, atomic and poll. Values are single-copy
// atomic 4- or 8-byte words, written and polled with relaxed gpu-scope
// accesses. Every wait is bounded: a wait that runs out marks the run failed
// (Ctl::bar_fail = 3, status TIMEOUT) and later waits give up at once.
__device__ __forceinline__ bool is_sentinel(double v) {
  return __double_as_longlong(v) == (long long)0x7ff4a5a5a5a5a5a5ull;
}
__device__ __forceinline__ bool is_sentinel(float v) { return __float_as_uint(v) == 0x7fa5a5a5u; }
template <typename T> __device__ __forceinline__ T sentinel_value() {
  if constexpr (sizeof(T) == 8) return __longlong_as_double((long long)0x7ff4a5a5a5a5a5a5ull);
  else return __uint_as_float(0x7fa5a5a5u);
}
__device__ __forceinline__ double ld_relaxed(const double *p) {
  double v;
  asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ float ld_relaxed(const float *p) {
  float v;
  asm volatile("ld.relaxed.gpu.global.f32 %0, [%1];" : "=f"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(double *p, double v) {
  asm volatile("st.relaxed.gpu.global.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed(float *p, float v) {
  asm volatile("st.relaxed.gpu.global.f32 [%0], %1;" ::"l"(p), "f"(v) : "memory");
}
// Bounded wait for one retry round of a batch of polled loads: returns false
// (and marks the run failed) when the wait ran out or another wait already
// failed.
__device__ __forceinline__ bool poll_again(Ctl *ctl, unsigned int &spins) {
  if (++spins > kBarrierSpins || ((spins & 255) == 0 && *(volatile int *)&ctl->bar_fail)) {
    if (!*(volatile int *)&ctl->bar_fail) {
      atomicExch(&ctl->bar_fail, 3);
      ctl->status = ST_TIMEOUT;
      __threadfence();
      atomicExch(&ctl->done, 1);
    }
    return false;
  }
  if (spins > 4) __nanosleep(32);
  return true;
}

// One staged row (thread per row, data in shared memory): the column
// indices come first so that all neighbour gathers of the row are in flight
// together. Same arithmetic as phase_row.
template <typename V, typename T>
__device__ __forceinline__ void staged_row(const Phase &P, int row, int lane, int w, const V *sv,
                                           const int *sc, const V *sd, const T *src, T *ybuf,
                                           T *hat, Ctl *ctl) {
  // gathers in flight per batch (8 in FP32 spilled once the ring's state
  // was added to the kernel)
  constexpr int SB = sizeof(T) == 8 ? 4 : 6;
  const T *own = P.own_y ? ybuf : src;
  const T *nbr = P.nbr_hat ? hat : ybuf;
  // only values of ybuf and hat can be sentinels: reads of the input src are
  // never checked (any bit pattern there is data)
  T a0, a1, a2;
  unsigned int spins = 0;
  do {   // all three again while any is still a sentinel
    a0 = ld_relaxed(own + 3 * row); a1 = ld_relaxed(own + 3 * row + 1);
    a2 = ld_relaxed(own + 3 * row + 2);
  } while (P.own_y && (is_sentinel(a0) || is_sentinel(a1) || is_sentinel(a2)) &&
           poll_again(ctl, spins));
  for (int k0 = 0; k0 < w; k0 += SB) {
    int c[SB];
    T y[SB][3];
#pragma unroll
    for (int j = 0; j < SB; ++j) c[j] = (k0 + j < w) ? sc[(k0 + j) * 32 + lane] : -1;
    bool wait;
    do {   // the whole batch again while any value is still a sentinel
      wait = false;
#pragma unroll
      for (int j = 0; j < SB; ++j)
        if (c[j] >= 0) {
          const T *xs = (c[j] < P.src_rows ? src : nbr) + 3 * c[j];
          y[j][0] = ld_relaxed(xs);
          y[j][1] = ld_relaxed(xs + 1);
          y[j][2] = ld_relaxed(xs + 2);
        }
#pragma unroll
      for (int j = 0; j < SB; ++j)
        if (c[j] >= P.src_rows)
          wait |= is_sentinel(y[j][0]) || is_sentinel(y[j][1]) || is_sentinel(y[j][2]);
    } while (wait && poll_again(ctl, spins));
#pragma unroll
    for (int j = 0; j < SB; ++j)
      if (c[j] >= 0) {
        V b[9];
        load_block<V, false>(sv + (size_t)(k0 + j) * 9 * 32, lane, b);
        a0 = fma(-(T)b[0], y[j][0], a0); a0 = fma(-(T)b[1], y[j][1], a0);
        a0 = fma(-(T)b[2], y[j][2], a0);
        a1 = fma(-(T)b[3], y[j][0], a1); a1 = fma(-(T)b[4], y[j][1], a1);
        a1 = fma(-(T)b[5], y[j][2], a1);
        a2 = fma(-(T)b[6], y[j][0], a2); a2 = fma(-(T)b[7], y[j][1], a2);
        a2 = fma(-(T)b[8], y[j][2], a2);
      }
  }
  if (P.has_d) apply_dp<V, T, false>(sd, lane, a0, a1, a2);
  if (P.to_y) {
    st_relaxed(ybuf + 3 * row, a0); st_relaxed(ybuf + 3 * row + 1, a1);
    st_relaxed(ybuf + 3 * row + 2, a2);
    if (row < P.final0) return;
    if (P.final_d) apply_dp<V, T, false>(sd, lane, a0, a1, a2);
  }
  st_relaxed(hat + 3 * row, a0); st_relaxed(hat + 3 * row + 1, a1); st_relaxed(hat + 3 * row + 2, a2);
}

// Component c of one staged row: own_c - sum_k B_k[c,:] y_k with the FMA
// sequence of that component in staged_row, so a row whose three components
// are computed by three warps gets the same bits.
template <typename V, typename T>
__device__ __forceinline__ T staged_comp(const Phase &P, int c, int row, int lane, int w,
                                         const V *sv, const int *sc, const T *src, const T *ybuf,
                                         const T *hat, Ctl *ctl) {
  constexpr int SB = sizeof(T) == 8 ? 4 : 8;
  const T *own = P.own_y ? ybuf : src;
  const T *nbr = P.nbr_hat ? hat : ybuf;
  T a;
  unsigned int spins = 0;
  do {   // (src is never checked: see staged_row)
    a = ld_relaxed(own + 3 * row + c);
  } while (P.own_y && is_sentinel(a) && poll_again(ctl, spins));
  for (int k0 = 0; k0 < w; k0 += SB) {
    int cc[SB];
    T y[SB][3];
#pragma unroll
    for (int j = 0; j < SB; ++j) cc[j] = (k0 + j < w) ? sc[(k0 + j) * 32 + lane] : -1;
    bool wait;
    do {   // the whole batch again while any value is still a sentinel
      wait = false;
#pragma unroll
      for (int j = 0; j < SB; ++j)
        if (cc[j] >= 0) {
          const T *xs = (cc[j] < P.src_rows ? src : nbr) + 3 * cc[j];
          y[j][0] = ld_relaxed(xs);
          y[j][1] = ld_relaxed(xs + 1);
          y[j][2] = ld_relaxed(xs + 2);
        }
#pragma unroll
      for (int j = 0; j < SB; ++j)
        if (cc[j] >= P.src_rows)
          wait |= is_sentinel(y[j][0]) || is_sentinel(y[j][1]) || is_sentinel(y[j][2]);
    } while (wait && poll_again(ctl, spins));
#pragma unroll
    for (int j = 0; j < SB; ++j)
      if (cc[j] >= 0) {
        const V *b = sv + (size_t)(k0 + j) * 9 * 32;
        a = fma(-(T)b[sl_idx<V>(0, 3 * c, lane)], y[j][0], a);
        a = fma(-(T)b[sl_idx<V>(0, 3 * c + 1, lane)], y[j][1], a);
        a = fma(-(T)b[sl_idx<V>(0, 3 * c + 2, lane)], y[j][2], a);
      }
  }
  return a;
}

// Warps per CTA of the single-launch apply that work in groups of three on
// the FP64 staged steps (one warp per row component)
template <typename T> __host__ __device__ constexpr int comp_groups() {
  return coop_threads<T>() / 32 / 3;
}

// The three warps of component group g (named barrier 1 + g; 0 is
// __syncthreads)
__device__ __forceinline__ void group_sync(int g) {
  asm volatile("bar.sync %0, 96;" ::"r"(1 + g) : "memory");
}

#ifndef GBILU_LARGE_CACHED
#define GBILU_LARGE_CACHED 1
#endif
#ifndef GBILU_DYNAMIC_LARGE
#define GBILU_DYNAMIC_LARGE 1
#endif
#ifndef GBILU_DYN_MIN_ROUNDS
#define GBILU_DYN_MIN_ROUNDS 1LL
#endif
#ifndef GBILU_DYN_FIRST_STATIC
#define GBILU_DYN_FIRST_STATIC 1
#endif
#ifndef GBILU_DYN_MAX_ROUNDS
#define GBILU_DYN_MAX_ROUNDS (1LL << 30)
#endif
// Large steps: each warp asks L2 for the matrix slice it (or, with the
// dynamic order, another warp) will take this many rounds of the grid's
// warps ahead, by one bulk prefetch per array; 0 turns it off.
#ifndef GBILU_L2_PREFETCH
#define GBILU_L2_PREFETCH 0
#endif
// Vector loads of the large steps go through L1. Every large step follows a
// grid barrier whose acquire (ld.acquire.gpu, then the CTA barrier) orders
// the earlier steps' writes from other SMs before these loads, and no row a
// large step reads is written during it (rows of one color are not
// coupled), so the SM's L1 cannot serve a stale value; the three components
// of a neighbour and neighbours shared by nearby rows then cost one L2
// sector fetch instead of one per load.
constexpr bool kLargeCached = GBILU_LARGE_CACHED != 0;
template <typename T> __device__ __forceinline__ T ldl(const T *p) {
  if (kLargeCached) return __ldca(p);
  return __ldcg(p);
}

// Bounded mbarrier phase wait of the ring. Gives up after kStageSpins
// polls, or early once another wait of the run failed. A parity wait only
// tells the current phase of a barrier from the one before it, so a waiter
// must never be two phases ahead: the producer waits for the phases of a
// stage's free barrier one after another, and a compute warp first waits
// until the stage's sequence word names its slice (the producer writes it
// only once the previous round of that stage was consumed, hence filled),
// then for the fill itself.
__device__ __forceinline__ bool ring_wait(Ctl *ctl, uint64_t *bar, uint32_t parity) {
  unsigned int spins = 0;
  while (!mbar_try_wait(bar, parity)) {
    if (++spins > kStageSpins || ((spins & 1023) == 0 && *(volatile int *)&ctl->bar_fail))
      return false;
  }
  return true;
}

__device__ __forceinline__ bool ring_wait_slice(Ctl *ctl, const unsigned int *seq, unsigned int g,
                                                uint64_t *bar, uint32_t parity) {
  unsigned int spins = 0;
  while (*(volatile const unsigned int *)seq != g) {
    if (++spins > kStageSpins || ((spins & 1023) == 0 && *(volatile int *)&ctl->bar_fail))
      return false;
    if (spins > 64) __nanosleep(32);
  }
  return ring_wait(ctl, bar, parity);
}

// Producer of the ring, one lane per stage: the CTA's slices of the
// streamed steps, numbered in launch order (the host lists them), and lane
// st of the producer warp fills stage st with the slices g = st (mod ns),
// each once the compute warp that held the slice g - ns released the
// stage. The warp stays converged: every pass each lane tests (without
// blocking) whether its stage is free and, if so, issues the fill and loads
// the slot range of its next slice. Before it returns every lane waits for
// its own last copies, so that the CTA never ends with a bulk copy in
// flight.
template <typename V>
__device__ void ring_produce(Ctl *ctl, const StagePlan &sp, unsigned char *ring, uint64_t *full,
                             uint64_t *empty, int *ring_w, unsigned int *ring_seq,
                             const int *off1, const int *col1, const V *val1, const int *off2,
                             const int *col2, const V *val2, const V *dmat, unsigned int st) {
  const unsigned int ns = (unsigned int)sp.ring_ns;
  const unsigned int total = (unsigned int)sp.ring_cnt[blockIdx.x];
  const unsigned int *tab = sp.ring_tab + (size_t)blockIdx.x * sp.ring_max;
  unsigned int g = st, k = 0;   // next slice of this lane, fills so far
  bool active = st < ns && g < total;
  unsigned int ent = 0;
  int o = 0, w = 0;
  auto load = [&]() {
    ent = __ldg(tab + g);
    const int *off = (ent >> 30) & 1u ? off2 : off1;
    const int sl = (int)(ent & 0x3fffffffu);
    o = __ldg(off + sl);
    w = __ldg(off + sl + 1) - o;
  };
  if (active) load();
  unsigned int spins = 0;
  bool ok = true;
  while (__any_sync(0xffffffffu, active)) {
    if (active) {
      if (k == 0 || mbar_test_wait(&empty[st], (k - 1) & 1u)) {
        const int sl = (int)(ent & 0x3fffffffu);
        const bool m2 = (ent >> 30) & 1u;
        const int *col = m2 ? col2 : col1;
        const V *val = m2 ? val2 : val1;
        const uint32_t vb = (uint32_t)(w * 9 * 32 * sizeof(V)), cb = (uint32_t)(w * 32 * sizeof(int));
        const uint32_t db = (ent >> 31) ? (uint32_t)(9 * 32 * sizeof(V)) : 0u;
        unsigned char *dst = ring + (size_t)st * sp.ring_stride;
        ring_w[st] = w;
        // the slice number: a compute warp waits for it before the fill
        *(volatile unsigned int *)&ring_seq[st] = g;
        mbar_expect_tx(&full[st], vb + cb + db);   // this lane's arrival, released to the waiters
        if (vb) bulk_g2s(dst, val + (size_t)o * 9 * 32, vb, &full[st]);
        if (cb) bulk_g2s(dst + vb, col + (size_t)o * 32, cb, &full[st]);
        if (db) bulk_g2s(dst + vb + cb, dmat + (size_t)sl * 9 * 32, db, &full[st]);
        g += ns;
        ++k;
        spins = 0;
        active = g < total;
        if (active) load();
      } else if (++spins > kStageSpins ||
                 ((spins & 1023) == 0 && *(volatile int *)&ctl->bar_fail)) {
        active = false;
        ok = false;
      }
    }
  }
  if (!ok && !*(volatile int *)&ctl->bar_fail) mark_stage_timeout(ctl);
  // the last fill of this stage: wait (bounded) for its bytes
  if (st < ns && k > 0) ring_wait(ctl, &full[st], (k - 1) & 1u);
}

// One row of a streamed slice: the same arithmetic as phase_row (blocks in
// slot order, three FMAs per block row entry, then phase_store), with the
// slice's values, column indices and D block read from the ring stage.
template <typename V, typename T>
__device__ __forceinline__ void ring_row(const Phase &P, int row, int lane, int w, const V *sv,
                                         const int *sc, const V *sd, const T *src, T *ybuf,
                                         T *hat) {
  // gathers in flight per batch (within the kernel's 128 registers)
  constexpr int B = sizeof(T) == 8 ? 2 : 4;
  const T *own = P.own_y ? ybuf : src;
  const T *nbr = P.nbr_hat ? hat : ybuf;
  T a0 = ldl(own + 3 * row), a1 = ldl(own + 3 * row + 1), a2 = ldl(own + 3 * row + 2);
  for (int k0 = 0; k0 < w; k0 += B) {
    int c[B];
    T x[B][3];
#pragma unroll
    for (int j = 0; j < B; ++j) c[j] = (k0 + j < w) ? sc[(k0 + j) * 32 + lane] : -1;
#pragma unroll
    for (int j = 0; j < B; ++j)
      if (c[j] >= 0) {
        const T *xs = (c[j] < P.src_rows ? src : nbr) + 3 * c[j];
        x[j][0] = ldl(xs);
        x[j][1] = ldl(xs + 1);
        x[j][2] = ldl(xs + 2);
      }
#pragma unroll
    for (int j = 0; j < B; ++j)
      if (c[j] >= 0) {
        V b[9];
        load_block<V, false>(sv + (size_t)(k0 + j) * 9 * 32, lane, b);
        a0 = fma(-(T)b[0], x[j][0], a0); a0 = fma(-(T)b[1], x[j][1], a0);
        a0 = fma(-(T)b[2], x[j][2], a0);
        a1 = fma(-(T)b[3], x[j][0], a1); a1 = fma(-(T)b[4], x[j][1], a1);
        a1 = fma(-(T)b[5], x[j][2], a1);
        a2 = fma(-(T)b[6], x[j][0], a2); a2 = fma(-(T)b[7], x[j][1], a2);
        a2 = fma(-(T)b[8], x[j][2], a2);
      }
  }
  phase_store<V, T, false>(P, row, sd, lane, a0, a1, a2, ybuf, hat);
}

// hat = M^-1 src (or M^-T src): all color steps of the L and U sweeps in one
// launch. Consecutive steps are separated by a grid barrier, by a CTA
// barrier (two single-slice steps on CTA 0), or by nothing at all inside a
// run of staged steps, whose consumers wait for the values they read
// (sentinel outputs, see is_sentinel). Vector loads go through
// L2 because earlier steps of the same launch wrote them on other SMs.
// Staged small steps read their matrix data from shared memory; with a
// ring (sp.ring_ns > 0) the last warp becomes the producer of the large
// steps' slices and the other warps compute, synchronising among
// themselves on a named barrier.
template <typename V, typename T>
__global__ void __launch_bounds__(coop_threads<T>(), 1)
k_ilu_coop(Ctl *ctl, PhaseList ph, StagePlan sp, const int *__restrict__ off1,
           const int *__restrict__ col1, const V *__restrict__ val1, const int *__restrict__ off2,
           const int *__restrict__ col2, const V *__restrict__ val2, const V *__restrict__ dmat,
           const T *src, T *ybuf, T *hat) {
  extern __shared__ __align__(128) unsigned char stage_smem[];
  __shared__ uint64_t stage_bar;
  __shared__ uint64_t ring_full[kRingMax], ring_empty[kRingMax];
  __shared__ int ring_w[kRingMax];
  __shared__ unsigned int ring_seq[kRingMax];   // slice number a stage is filled with
  __shared__ StageEntry stage_tab[kMaxStage];
  __shared__ int stage_n;
  __shared__ T xch[sizeof(T) == 8 ? comp_groups<T>() : 1][3][32];   // FP64 component exchange
  if (ctl->done) return;
  constexpr int NT = coop_threads<T>();
  const bool ring = sp.ring_ns > 0;
  const int ncw = ring ? NT / 32 - 1 : NT / 32;   // compute warps
  const int nct = 32 * ncw;                       // compute threads
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  bool staged_ready = false;
  if (ring && threadIdx.x == 0) {
    for (int st = 0; st < sp.ring_ns; ++st) {
      mbar_init(&ring_full[st], 1);
      mbar_init(&ring_empty[st], 1);
      ring_seq[st] = 0xffffffffu;
    }
  }
  if (sp.enabled) {
    const int2 cnt = sp.cnt[blockIdx.x];
    if (threadIdx.x == 0) {
      stage_n = cnt.x;
      mbar_init(&stage_bar, 1);
      mbar_expect_tx(&stage_bar, (uint32_t)cnt.y);
    }
    if (threadIdx.x < cnt.x) stage_tab[threadIdx.x] = sp.tab[(size_t)blockIdx.x * kMaxStage + threadIdx.x];
  }
  __syncthreads();
  if (sp.enabled) {
    if (threadIdx.x < stage_n) {
      const StageEntry e = stage_tab[threadIdx.x];
      const Phase P = ph.p[e.q];
      const int s = P.slice0 + e.j;
      const int *off = P.mat ? off2 : off1;
      const int *col = P.mat ? col2 : col1;
      const V *val = P.mat ? val2 : val1;
      const size_t o = (size_t)__ldg(off + s);
      unsigned char *dst = stage_smem + e.pos;
      const uint32_t vb = (uint32_t)(e.w * 9 * 32 * sizeof(V)), cb = (uint32_t)(e.w * 32 * sizeof(int));
      if (vb) bulk_g2s(dst, val + o * 9 * 32, vb, &stage_bar);
      if (cb) bulk_g2s(dst + vb, col + o * 32, cb, &stage_bar);
      if (P.uses_d())
        bulk_g2s(dst + vb + cb, dmat + (size_t)s * 9 * 32, (uint32_t)(9 * 32 * sizeof(V)), &stage_bar);
    }
    // sentinels into the outputs of this CTA's staged rows; a grid barrier
    // separates them from every consumer
    const T sent = sentinel_value<T>();
    for (int e = warp; e < stage_n; e += NT / 32) {
      const StageEntry E = stage_tab[e];
      const Phase &P = ph.p[E.q];
      const int r = 32 * E.j + lane;
      if (r >= P.nrows) continue;
      const int row = P.row0 + r;
      if (P.to_y)
        for (int k = 0; k < 3; ++k) st_relaxed(ybuf + 3 * row + k, sent);
      if (!P.to_y || row >= P.final0)
        for (int k = 0; k < 3; ++k) st_relaxed(hat + 3 * row + k, sent);
    }
  }
  // the slice counters of the large steps after the first: cleared here,
  // before this CTA's first grid barrier, so before any of those steps
  // starts; the first step keeps the static assignment
  if (GBILU_DYNAMIC_LARGE && blockIdx.x == 0 && threadIdx.x < ph.n && threadIdx.x > 0)
    ctl->step_next[threadIdx.x] = 0u;
  unsigned char *ring_base = stage_smem + sp.ring_off;
  if (ring && warp == NT / 32 - 1) {
    // the producer warp (one lane per stage) leaves the CTA's barriers
    // from here on
    ring_produce<V>(ctl, sp, ring_base, ring_full, ring_empty, ring_w, ring_seq, off1, col1,
                    val1, off2, col2, val2, dmat, (unsigned int)lane);
    return;
  }
  const int stride = gridDim.x * nct;
  // Every thread acquires the completed bulk copies itself, with a bounded
  // wait, just before the grid barrier that precedes the first staged step
  // (the copies finished long before); the barrier's own CTA-wide sync
  // then makes a wait that ran out a failure of the whole CTA.
  int first_staged = ph.n;
  if (sp.enabled)
    for (int q = 0; q < ph.n; ++q)
      if (ph.p[q].staged) { first_staged = q; break; }
  auto copies_late = [&]() {
    unsigned int spins = 0;
    while (!mbar_try_wait(&stage_bar, 0))
      if (++spins > kStageSpins) return true;
    return false;
  };
  bool run = true;
  if (first_staged == 0) {
    // every step is small: the sentinels need a grid barrier before any step
    run = grid_barrier(ctl, copies_late(), nct);
    staged_ready = run;
  }
  unsigned int gseq = 0;   // ring slices of this CTA in the streamed steps so far
  for (int q = 0; run && q < ph.n; ++q) {
    if (ph.trace && blockIdx.x == 0 && threadIdx.x == 0) ctl->phase_ns[q] = globaltimer();
    const Phase P = ph.p[q];
    const int *off = P.mat ? off2 : off1;
    const int *col = P.mat ? col2 : col1;
    const V *val = P.mat ? val2 : val1;
    bool late = false;   // a ring wait of this warp ran out
    if (P.staged && sp.enabled) {
      if constexpr (sizeof(T) == 8) {
        // FP64: three warps per slice, one per row component. A small step
        // gives each SM one or two slices, and one warp's FP64 instructions
        // issue at one per 64 cycles whatever the number of active lanes,
        // so a slice's 9 FMA per block on one warp is the step's critical
        // path; split by component it is a third of that. The entries of a
        // step are contiguous in the CTA's table (the host adds them step
        // by step).
        constexpr int G = comp_groups<T>();
        const int grp = warp / 3, c = warp - 3 * grp;
        int e0 = 0;
        while (e0 < stage_n && stage_tab[e0].q < q) ++e0;
        int e1 = e0;
        while (e1 < stage_n && stage_tab[e1].q == q) ++e1;
        for (int base = e0; base < e1; base += G) {
          const int e = base + grp;
          const bool act = grp < G && e < e1;
          bool valid = false;
          int row = 0;
          T a = 0;
          const V *sd = nullptr;
          if (act) {
            const StageEntry E = stage_tab[e];
            const int r = 32 * E.j + lane;
            valid = r < P.nrows;
            row = P.row0 + r;
            const V *sv = reinterpret_cast<const V *>(stage_smem + E.pos);
            const int *sc =
                reinterpret_cast<const int *>(stage_smem + E.pos + E.w * 9 * 32 * sizeof(V));
            sd = reinterpret_cast<const V *>(stage_smem + E.pos + E.w * 9 * 32 * sizeof(V) +
                                             E.w * 32 * sizeof(int));
            if (valid) a = staged_comp<V, T>(P, c, row, lane, E.w, sv, sc, src, ybuf, hat, ctl);
          }
          if (!act) continue;   // the whole group (same e) skips the round
          // the D products need all three components: the group's warps
          // exchange them through shared memory, synchronised by the group's
          // own named barrier (warps of other groups may be in other steps)
          if (P.has_d) {
            xch[grp][c][lane] = a;
            group_sync(grp);
            if (valid)
              a = dot3<T>((T)sd[sl_idx<V>(0, 3 * c, lane)], (T)sd[sl_idx<V>(0, 3 * c + 1, lane)],
                          (T)sd[sl_idx<V>(0, 3 * c + 2, lane)], xch[grp][0][lane],
                          xch[grp][1][lane], xch[grp][2][lane]);
            group_sync(grp);
          }
          bool fin = true;
          if (P.to_y) {
            if (valid) st_relaxed(ybuf + 3 * row + c, a);
            fin = row >= P.final0;
            if (P.final_d) {
              xch[grp][c][lane] = a;
              group_sync(grp);
              if (valid && fin)
                a = dot3<T>((T)sd[sl_idx<V>(0, 3 * c, lane)], (T)sd[sl_idx<V>(0, 3 * c + 1, lane)],
                            (T)sd[sl_idx<V>(0, 3 * c + 2, lane)], xch[grp][0][lane],
                            xch[grp][1][lane], xch[grp][2][lane]);
              group_sync(grp);
            }
          }
          if (valid && fin) st_relaxed(hat + 3 * row + c, a);
        }
      } else {
        for (int e = warp; e < stage_n; e += ncw) {
          const StageEntry E = stage_tab[e];
          if (E.q != q) continue;
          const int r = 32 * E.j + lane;
          if (r >= P.nrows) continue;
          const V *sv = reinterpret_cast<const V *>(stage_smem + E.pos);
          const int *sc =
              reinterpret_cast<const int *>(stage_smem + E.pos + E.w * 9 * 32 * sizeof(V));
          const V *sd = reinterpret_cast<const V *>(stage_smem + E.pos + E.w * 9 * 32 * sizeof(V) +
                                                    E.w * 32 * sizeof(int));
          staged_row<V, T>(P, P.row0 + r, lane, E.w, sv, sc, sd, src, ybuf, hat, ctl);
        }
      }
    } else if (P.streamed && ring) {
      // this CTA's slices j = blockIdx.x + t * grid come from the ring in
      // order; compute warp w takes the slices whose number in the CTA's
      // sequence is w modulo the compute warps
      const int nsl = (P.nrows + 31) >> 5;
      const int nq = (int)blockIdx.x < nsl ? (nsl - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
      const unsigned int ns = (unsigned int)sp.ring_ns;
      for (int t = (warp - (int)(gseq % ncw) + ncw) % ncw; t < nq; t += ncw) {
        const unsigned int g = gseq + t, st = g % ns;
        // every lane acquires the fill itself; the warp goes on only if all did
        const bool got = __all_sync(
            0xffffffffu, ring_wait_slice(ctl, &ring_seq[st], g, &ring_full[st], (g / ns) & 1u));
        if (!got) {
          // the other waits of the run give up at once from here on
          if (!*(volatile int *)&ctl->bar_fail) mark_stage_timeout(ctl);
          late = true;
          break;
        }
        const int j = blockIdx.x + t * gridDim.x;
        const int r = 32 * j + lane;
        const unsigned char *stage = ring_base + (size_t)st * sp.ring_stride;
        const int w = ring_w[st];
        if (r < P.nrows)
          ring_row<V, T>(P, P.row0 + r, lane, w, reinterpret_cast<const V *>(stage),
                         reinterpret_cast<const int *>(stage + w * 9 * 32 * sizeof(V)),
                         reinterpret_cast<const V *>(stage + w * 9 * 32 * sizeof(V) +
                                                     w * 32 * sizeof(int)),
                         src, ybuf, hat);
        __syncwarp();
        if (lane == 0) mbar_arrive(&ring_empty[st]);
      }
      gseq += nq;
    } else {
      const int nsl = (P.nrows + 31) >> 5;
      // Warp w of CTA b first takes slice w * grid + b (one round of the
      // grid's warps; slice j lands on CTA j % grid: the device numbering
      // puts a color's widest rows first, and contiguous chunks per CTA
      // would hand them all to the first CTAs, which every barrier then
      // waits for). Static: every further round the same way. dyn: the
      // slices after the first round are handed out in order by a counter,
      // so a warp that drew narrow slices takes more, each warp fetching
      // its next while it computes the current one. Only for steps after
      // the first with more slices than the grid has warps: a grid barrier
      // precedes each of them, CTA 0 cleared the counter before its first
      // grid barrier, and the one-slice steps that a CTA barrier links to a
      // neighbouring step keep their static owner.
      const long long nwt = stride >> 5;
      const bool dyn = GBILU_DYNAMIC_LARGE && q > 0 && nsl > 1 &&
                       nsl > GBILU_DYN_MIN_ROUNDS * nwt && nsl <= GBILU_DYN_MAX_ROUNDS * nwt;
      unsigned int *ctr = &ctl->step_next[q];
#if GBILU_L2_PREFETCH > 0
      // the first rounds here (lane k: round k of this warp's static
      // order), then round + GBILU_L2_PREFETCH of each slice taken
      const int nw = stride >> 5;
      const bool pd = P.uses_d();
      constexpr bool PF = sizeof(V) == 4;   // the FP64 steps are bound by the FP64 unit
      if (PF && lane < GBILU_L2_PREFETCH) {
        const int jp = warp * (int)gridDim.x + (int)blockIdx.x + lane * nw;
        if (jp < nsl) {
          const int o = off[P.slice0 + jp];
          prefetch_slice<V>(P.slice0 + jp, o, off[P.slice0 + jp + 1] - o, col, val, dmat, pd);
        }
      }
#endif
      int j = GBILU_DYN_FIRST_STATIC || !dyn
                  ? warp * (int)gridDim.x + (int)blockIdx.x
                  : __shfl_sync(0xffffffffu, lane == 0 ? (int)atomicAdd(ctr, 1u) : 0, 0);
      const int first_dyn = GBILU_DYN_FIRST_STATIC ? (int)nwt : 0;
      while (j < nsl) {
        const int jn =
            dyn ? (lane == 0 ? first_dyn + (int)atomicAdd(ctr, 1u) : 0) : j + (stride >> 5);
#if GBILU_L2_PREFETCH > 0
        // loaded now, the prefetch issued after this slice's row
        const int jp = j + GBILU_L2_PREFETCH * nw;
        const int po = PF && lane == 0 && jp < nsl ? off[P.slice0 + jp] : 0;
        const int pe = PF && lane == 0 && jp < nsl ? off[P.slice0 + jp + 1] : 0;
#endif
        const int t = 32 * j + lane;
        if (t < P.nrows)
          phase_row<V, T, !kLargeCached>(P, P.row0 + t, P.slice0 + j, lane, off, col, val, dmat,
                                         src, ybuf, hat);
#if GBILU_L2_PREFETCH > 0
        if (PF && lane == 0 && jp < nsl)
          prefetch_slice<V>(P.slice0 + jp, po, pe - po, col, val, dmat, pd);
#endif
        j = dyn ? __shfl_sync(0xffffffffu, jn, 0) : jn;
      }
    }
    bool ok = true;
    if (q + 1 < ph.n && P.flow_after && P.staged && ph.p[q + 1].staged && sp.enabled) {
      // data-ordered: the next step waits for the values it reads
    } else if (q + 1 < ph.n && P.local_after) {
      cta_sync(nct);   // the next step reads this one's rows, all written by this CTA
    } else if (q + 1 < ph.n) {
      const bool before_staged = q + 1 == first_staged;
      ok = grid_barrier(ctl, late || (before_staged && copies_late()), nct);
      if (ok && before_staged) staged_ready = true;
    } else if (late && !*(volatile int *)&ctl->bar_fail) {
      mark_stage_timeout(ctl);
    }
    if (ok && ph.trace && q + 1 == ph.n) {
      // the end of the last phase: after every CTA finished it
      ok = grid_barrier(ctl, false, nct);
      if (ok && blockIdx.x == 0 && threadIdx.x == 0) ctl->phase_ns[ph.n] = globaltimer();
    }
    if (!ok) break;
  }
  if (sp.enabled && !staged_ready) {
    // the copies were never acquired (a failed run): still wait, bounded,
    // for them before the CTA exits
    for (unsigned int k = 0; k < kStageSpins && !mbar_try_wait(&stage_bar, 0); ++k) {}
  }
}

// Self-test of the bounded waits (failure detection without a GPU fault):
// mode 0, a grid barrier that one of the two CTAs never reaches; mode 1, a
// data-ordered load of a word that stays the sentinel. Both waits run out
// after their poll limit, mark the run failed (Ctl::bar_fail 1 or 3,
// status TIMEOUT) and return, leaving the context usable.
__global__ void k_wait_probe(Ctl *ctl, int mode, const double *word) {
  if (mode == 0) {
    if (blockIdx.x == 1) return;   // never arrives
    grid_barrier(ctl);
  } else if (blockIdx.x == 0 && threadIdx.x == 0) {
    unsigned int spins = 0;
    double v;
    do {
      v = ld_relaxed(word);
    } while (is_sentinel(v) && poll_again(ctl, spins));
  }
}

// --------------------------------------------------------------------------
// fused vector kernels (grid-stride over the n unknowns)
// --------------------------------------------------------------------------

// Steps 0/1 of the FP64 solve after y = A x0 (k_spmv PLAIN into r):
// r = b - y (the RESID epilogue's arithmetic), rt = p = r, rho = ||r||^2 and
// the stop tests of the start. Split from the SpMV so that b can still be in
// transit while A x0 is computed. perm non-null: b is in the input numbering
// (device row i reads input row perm[i], as k_gather).
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_init_resid(Ctl *ctl, int n, const T *__restrict__ b, const int *__restrict__ perm,
             T *__restrict__ r, T *__restrict__ rt, T *__restrict__ p, double *partials) {
  double d = 0.0;
  DF f = {0.f, 0.f};
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const int row = i / 3;
    const T v = (perm ? b[3 * perm[row] + (i - 3 * row)] : b[i]) - r[i];
    r[i] = v; rt[i] = v; p[i] = v;
    if (sizeof(T) == 8) d += (double)v * v; else df_add_prod(f, (float)v, (float)v);
  }
  if (sizeof(T) == 4) d = df_value(f);
  double vv[1] = {d}, tot[1];
  if (grid_sum<1>(vv, partials, &ctl->counter[0], tot) && threadIdx.x == 0)
    finish_init<T>(ctl, tot[0]);
}

// Inner solves of iterative refinement start from d = 0: r = rt = p = rhs,
// rho = ||rhs||^2 (step 1 without the SpMV of step 0).
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_init_rhs(Ctl *ctl, int n, const T *__restrict__ rhs, T *__restrict__ r,
           T *__restrict__ rt, T *__restrict__ p, T *__restrict__ x, double *partials) {
  double d = 0.0;
  DF f = {0.f, 0.f};
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const T v = rhs[i];
    r[i] = v; rt[i] = v; p[i] = v; x[i] = 0;
    if (sizeof(T) == 8) d += (double)v * v; else df_add_prod(f, (float)v, (float)v);
  }
  if (sizeof(T) == 4) d = df_value(f);
  double v[1] = {d}, tot[1];
  if (grid_sum<1>(v, partials, &ctl->counter[0], tot) && threadIdx.x == 0)
    finish_init<T>(ctl, tot[0]);
}

// Steps 6-8 without the x update (deferred to the second half): s = r - alpha v,
// ||s|| and the stop tests (solver.vhd:867-936, is_final_iter solver.vhd:557).
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_update_s(Ctl *ctl, int n, const T *__restrict__ r, const T *__restrict__ v,
           T *__restrict__ s, double *partials) {
  if (ctl->done) return;
  const T alpha = (T)ctl->alpha;
  double d = 0.0;
  DF f = {0.f, 0.f};
  const int stride = gridDim.x * kThreads;
  // 4 elements per trip: their loads are in flight together
  for (int i0 = blockIdx.x * kThreads + threadIdx.x; i0 < n; i0 += 4 * stride) {
    T rv[4], vv4[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + u * stride;
      if (i < n) { rv[u] = r[i]; vv4[u] = v[i]; }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + u * stride;
      if (i < n) {
        const T si = fma(-alpha, vv4[u], rv[u]);
        s[i] = si;
        if (sizeof(T) == 8) d += (double)si * si; else df_add_prod(f, (float)si, (float)si);
      }
    }
  }
  if (sizeof(T) == 4) d = df_value(f);
  double vv[1] = {d}, tot[1];
  if (grid_sum<1>(vv, partials, &ctl->counter[3], tot) && threadIdx.x == 0) {
    const double ns = sqrt(tot[0]);
    push_norm(ctl, ns);
    if (!finite(ns)) stop(ctl, ST_NONFINITE, 1);
    else if (!ctl->ru_mode && !(ns > ctl->bound)) stop(ctl, ST_OK, 1);
    else if (ctl->k == ctl->maxit) stop(ctl, ST_MAXIT, 1);
    else ctl->half = 2 * ctl->k + 1;
  }
}

// Steps 11-14: x += alpha p^ + omega s^ (both halves' updates in one pass),
// r = s - omega t, ||r||, rho' = (r, rt), beta = (rho'/rho)(alpha/omega).
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_update_r(Ctl *ctl, int n, T *__restrict__ x, const T *__restrict__ ph,
           const T *__restrict__ sh, const T *__restrict__ s, const T *__restrict__ t,
           const T *__restrict__ rt, T *__restrict__ r, double *partials) {
  if (ctl->done) return;
  const T alpha = (T)ctl->alpha, omega = (T)ctl->omega;
  double d1 = 0.0, d2 = 0.0;
  DF f1 = {0.f, 0.f}, f2 = {0.f, 0.f};
  const int stride = gridDim.x * kThreads;
  // 4 elements per trip: their loads are in flight together
  for (int i0 = blockIdx.x * kThreads + threadIdx.x; i0 < n; i0 += 4 * stride) {
    T xv[4], phv[4], shv[4], sv[4], tv[4], rtv[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + u * stride;
      if (i < n) {
        xv[u] = x[i]; phv[u] = ph[i]; shv[u] = sh[i]; sv[u] = s[i]; tv[u] = t[i]; rtv[u] = rt[i];
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + u * stride;
      if (i < n) {
        x[i] = fma(omega, shv[u], fma(alpha, phv[u], xv[u]));
        const T ri = fma(-omega, tv[u], sv[u]);
        r[i] = ri;
        if (sizeof(T) == 8) { d1 += (double)ri * ri; d2 += (double)ri * rtv[u]; }
        else { df_add_prod(f1, (float)ri, (float)ri); df_add_prod(f2, (float)ri, (float)rtv[u]); }
      }
    }
  }
  if (sizeof(T) == 4) { d1 = df_value(f1); d2 = df_value(f2); }
  double vv[2] = {d1, d2}, tot[2];
  if (grid_sum<2>(vv, partials, &ctl->counter[4], tot) && threadIdx.x == 0) {
    const double nr = sqrt(tot[0]);
    push_norm(ctl, nr);
    ctl->dots[3] = tot[1];
    if (!finite(nr)) { stop(ctl, ST_NONFINITE, 0); return; }
    if (ctl->ru_mode) {
      // the recursive residual of the FP32 iteration only schedules a
      // replacement; the stop is decided on the true FP64 residual
      if (!(nr > ctl->bound) || nr < ctl->ru_delta * ctl->rmax) ctl->ru = 1;
      ctl->rmax = fmax(ctl->rmax, nr);
    } else if (!(nr > ctl->bound)) {
      stop(ctl, ST_OK, 0);
      return;
    }
    const double rho_new = tot[1];
    const double beta = (rho_new / ctl->rho) * (ctl->alpha / ctl->omega);
    ctl->rho_prev = ctl->rho;
    ctl->rho = rho_new;
    ctl->beta = beta;
    if (ctl->omega == 0.0 || !finite(beta)) { stop(ctl, ST_BREAKDOWN, 0); return; }
    if (ctl->timeout_ns && globaltimer() - ctl->t_start > ctl->timeout_ns) {
      stop(ctl, ST_TIMEOUT, 0);
      return;
    }
    ctl->k += 1;
    ctl->half = 2 * ctl->k;
  }
}

// --------------------------------------------------------------------------
// mixed precision by residual replacement (reliable updates)
// --------------------------------------------------------------------------

// Start of a mixed solve, after the FP64 residual r64 = b - A x (k_spmv
// RESID, which set norm0 and the bound): the FP32 iteration works on
// r64 / sigma with sigma = ||r64||; correction xc = 0.
__global__ void __launch_bounds__(kThreads)
k_ru_init(Ctl *ctl, int n, double delta, const double *__restrict__ r64,
          float *__restrict__ r, float *__restrict__ rt, float *__restrict__ p,
          float *__restrict__ xc, double *partials) {
  if (ctl->done) return;
  const double inv = 1.0 / ctl->norm0;
  DF f = {0.f, 0.f};
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const float v = (float)(r64[i] * inv);
    r[i] = v; rt[i] = v; p[i] = v; xc[i] = 0.f;
    df_add_prod(f, v, v);
  }
  double vv[1] = {df_value(f)}, tot[1];
  if (grid_sum<1>(vv, partials, &ctl->counter[6], tot) && threadIdx.x == 0) {
    ctl->ru_mode = 1;
    ctl->ru_delta = delta;
    ctl->sigma = ctl->norm0;
    ctl->rho = tot[0];
    ctl->rmax = sqrt(tot[0]);
    ctl->true_norm = ctl->norm0;
    ctl->bound = ctl->bound / ctl->sigma;   // recursive norms are in units of sigma
  }
}

// Replacement, part 1: x64 += sigma * xc, xc = 0 (the FP32 correction
// accumulated since the last replacement goes into the FP64 solution).
__global__ void __launch_bounds__(kThreads)
k_ru_accumulate(const Ctl *ctl, int n, float *__restrict__ xc, double *__restrict__ x64,
                int always) {
  if (!always && (!ctl->ru || ctl->done)) return;
  const double sg = ctl->sigma;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    x64[i] = fma(sg, (double)xc[i], x64[i]);
    xc[i] = 0.f;
  }
}

// Replacement, part 3 (after r64 = b - A x64 by k_spmv in TRUE mode):
// r = r64 / sigma; the true norm decides the stop; otherwise the FP32
// iteration continues from the replaced residual with rho' = (r, rt) and
// beta recomputed from it.
__global__ void __launch_bounds__(kThreads)
k_ru_replace(Ctl *ctl, int n, const double *__restrict__ r64, float *__restrict__ r,
             const float *__restrict__ rt, double *partials) {
  if (!ctl->ru || ctl->done) return;
  const double inv = 1.0 / ctl->sigma;
  DF f1 = {0.f, 0.f}, f2 = {0.f, 0.f};
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const float v = (float)(r64[i] * inv);
    r[i] = v;
    df_add_prod(f1, v, v);
    df_add_prod(f2, v, rt[i]);
  }
  double vv[2] = {df_value(f1), df_value(f2)}, tot[2];
  if (grid_sum<2>(vv, partials, &ctl->counter[7], tot) && threadIdx.x == 0) {
    ctl->ru = 0;
    ctl->replacements += 1;
    const double tn = ctl->true_norm;          // set by the TRUE-mode SpMV
    push_norm(ctl, tn / ctl->sigma);
    if (!finite(tn)) { stop(ctl, ST_NONFINITE, 0); return; }
    if (!(tn / ctl->sigma > ctl->bound)) { stop(ctl, ST_OK, 0); return; }
    const double rho_new = tot[1];
    ctl->beta = (rho_new / ctl->rho_prev) * (ctl->alpha / ctl->omega);
    ctl->rho = rho_new;
    ctl->rmax = sqrt(tot[0]);
    if (!finite(ctl->beta)) stop(ctl, ST_BREAKDOWN, 0);
  }
}

// Steps 15-17 (update_p, vector_ops.vhd:429-434): p = r + beta (p - omega v).
// Also drives the graph's while loop.
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_update_p(Ctl *ctl, int n, const T *__restrict__ r, const T *__restrict__ v,
           T *__restrict__ p, unsigned long long cond) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl->body_runs += 1;
    // hard stop as a second guard: the loop can never run past maxit + 1
    if (cond)
      cudaGraphSetConditional((cudaGraphConditionalHandle)cond,
                              (ctl->done || ctl->body_runs > ctl->maxit + 1) ? 0u : 1u);
  }
  if (ctl->done) return;
  const T beta = (T)ctl->beta, omega = (T)ctl->omega;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    const T pi = fma(beta, fma(-omega, v[i], p[i]), r[i]);
    p[i] = pi;
  }
}

// After the loop: a stop after a first half still owes x += alpha p^.
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_finish_x(const Ctl *ctl, int n, T *__restrict__ x, const T *__restrict__ ph) {
  if (!ctl->stop_half) return;
  const T alpha = (T)ctl->alpha;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads)
    x[i] = fma(alpha, ph[i], x[i]);
}

// --------------------------------------------------------------------------
// permutation, precision conversion, refinement and gradient kernels
// --------------------------------------------------------------------------

// out[3i+r] = in[3 perm[i] + r]  (original -> permuted numbering); nz (may
// be null) is set when any value is not zero
template <typename TI, typename TO>
__global__ void k_gather(int nb, const int *__restrict__ perm, const TI *__restrict__ in,
                         TO *__restrict__ out, double scale, int *nz = nullptr) {
  bool any = false;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < 3 * nb; i += gridDim.x * kThreads) {
    const int b = i / 3, r = i - 3 * b;
    const TI v = in[3 * perm[b] + r];
    any |= v != (TI)0;
    out[i] = (TO)((double)v * scale);
  }
  if (nz && __syncthreads_or(any) && threadIdx.x == 0) *nz = 1;
}

// out[3 perm[i] + r] = in[3i+r]  (permuted -> original numbering); nz as
// for k_gather
template <typename T>
__global__ void k_scatter(int nb, const int *__restrict__ perm, const T *__restrict__ in,
                          T *__restrict__ out, int *nz = nullptr) {
  bool any = false;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < 3 * nb; i += gridDim.x * kThreads) {
    const int b = i / 3, r = i - 3 * b;
    const T v = in[i];
    any |= v != (T)0;
    out[3 * perm[b] + r] = v;
  }
  if (nz && __syncthreads_or(any) && threadIdx.x == 0) *nz = 1;
}

// out = (float)(scale * in): the FP32 right-hand side of a refinement step
__global__ void k_scale_convert(int n, double scale, const double *__restrict__ in,
                                float *__restrict__ out) {
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads)
    out[i] = (float)(scale * in[i]);
}

// x += scale * d (FP64 x, FP32 correction of one refinement step)
__global__ void k_axpy_f2d(int n, double scale, const float *__restrict__ d,
                           double *__restrict__ x) {
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads)
    x[i] = fma(scale, (double)d[i], x[i]);
}

// ||v||^2 into ctl->dots[0] (refinement residual norm), FP64
__global__ void __launch_bounds__(kThreads)
k_norm2(Ctl *ctl, int n, const double *__restrict__ v, double *partials) {
  double d = 0.0;
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads)
    d += v[i] * v[i];
  double vv[1] = {d}, tot[1];
  if (grid_sum<1>(vv, partials, &ctl->counter[5], tot) && threadIdx.x == 0)
    ctl->dots[0] = tot[0];
}

// (x, y) of FP32 vectors into ctl->dots[0] two ways: mode 0 as the FP32
// kernels of the solve accumulate their dots (a double-float sum per thread
// on the FP32 pipe, FP64 across threads), mode 1 with an FP64 sum per
// thread (a diagnostic of the first against the second).
__global__ void __launch_bounds__(kThreads)
k_dot_check(Ctl *ctl, int n, const float *__restrict__ x, const float *__restrict__ y, int mode,
            double *partials) {
  double d = 0.0;
  DF f = {0.f, 0.f};
  for (int i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    if (mode == 0) df_add_prod(f, x[i], y[i]);
    else d += (double)x[i] * (double)y[i];
  }
  if (mode == 0) d = df_value(f);
  double v[1] = {d}, tot[1];
  if (grid_sum<1>(v, partials, &ctl->counter[5], tot) && threadIdx.x == 0) ctl->dots[0] = tot[0];
}

// dA[b] = -lambda_i x_j^T for every block b = (i, j) of the pattern in the
// input numbering and block order (the pattern gradient of L(x(A)),
// x = A^-1 b; brow[b], col[b]: the block's row and column). One thread per
// entry, in dA's order, so the 72 bytes written per block stream out in
// order; lambda and x are read in the input numbering. (A thread per
// permuted row spread each store over 32 cache lines, a warp per row waited
// on a chain of dependent loads, a thread per entry of the permuted pattern
// wrote scattered blocks: 1.44, 0.51 and 0.47 ms for the 2M-cell system.)
__global__ void __launch_bounds__(kThreads)
k_grad_a(long long nnzb, const int *__restrict__ brow, const int *__restrict__ col,
         const double *__restrict__ lam, const double *__restrict__ x, double *__restrict__ dA) {
  const long long n = 9 * nnzb;
  for (long long t = blockIdx.x * (long long)kThreads + threadIdx.x; t < n;
       t += (long long)gridDim.x * kThreads) {
    const long long b = t / 9;
    const int e = (int)(t - 9 * b);
    dA[t] = -lam[3 * brow[b] + e / 3] * x[3 * col[b] + e % 3];
  }
}

// --------------------------------------------------------------------------
// block ILU(0) on the device
// --------------------------------------------------------------------------

// Every product and sum below is an explicitly rounded IEEE operation in the
// same order as the host factorization (gbilu_host.cpp), with no fused
// multiply-add, so the device factors equal the host ones bit for bit.
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }

__device__ __forceinline__ void mul3_exact(const double *a, const double *b, double *o) {
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c)
      o[r * 3 + c] = dadd(dadd(dmul(a[r * 3], b[c]), dmul(a[r * 3 + 1], b[3 + c])),
                          dmul(a[r * 3 + 2], b[6 + c]));
}

// 3x3 inverse by cofactors; false when the block is singular or not finite
__device__ __forceinline__ bool inv3_exact(const double *a, double *o) {
  const double c00 = dsub(dmul(a[4], a[8]), dmul(a[5], a[7]));
  const double c01 = dsub(dmul(a[5], a[6]), dmul(a[3], a[8]));
  const double c02 = dsub(dmul(a[3], a[7]), dmul(a[4], a[6]));
  const double det = dadd(dadd(dmul(a[0], c00), dmul(a[1], c01)), dmul(a[2], c02));
  if (det == 0.0 || !isfinite(det)) return false;
  const double id = __ddiv_rn(1.0, det);
  o[0] = dmul(c00, id);
  o[1] = dmul(dsub(dmul(a[2], a[7]), dmul(a[1], a[8])), id);
  o[2] = dmul(dsub(dmul(a[1], a[5]), dmul(a[2], a[4])), id);
  o[3] = dmul(c01, id);
  o[4] = dmul(dsub(dmul(a[0], a[8]), dmul(a[2], a[6])), id);
  o[5] = dmul(dsub(dmul(a[2], a[3]), dmul(a[0], a[5])), id);
  o[6] = dmul(c02, id);
  o[7] = dmul(dsub(dmul(a[1], a[6]), dmul(a[0], a[7])), id);
  o[8] = dmul(dsub(dmul(a[0], a[4]), dmul(a[1], a[3])), id);
  return true;
}

// pv[k] = vals[src[k]] (input order -> color-permuted order), 9 per block
__global__ void k_permute_blocks(int nnzb, const int *__restrict__ src,
                                 const double *__restrict__ vals, double *__restrict__ pv) {
  for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < 9LL * nnzb;
       i += (long long)gridDim.x * kThreads) {
    const long long k = i / 9, e = i - 9 * k;
    pv[i] = vals[(long long)src[k] * 9 + e];
  }
}

// IKJ block ILU(0) of the rows of one color (rows of one color are never
// coupled, and all earlier colors are final): for each k < i in row i,
// L_ik = A_ik U_kk^-1, then A_ij -= L_ik U_kj for the j > k present in both
// rows (a merge of the two sorted column lists); D_i^-1 = inv(A_ii).
// A singular pivot records the smallest failing row in *bad.
__global__ void k_bilu0_color(int row0, int nrows, const int *__restrict__ rp,
                              const int *__restrict__ ci, const int *__restrict__ diag,
                              double *v, double *dinv, int *bad) {
  const int t = blockIdx.x * kThreads + threadIdx.x;
  if (t >= nrows) return;
  const int i = row0 + t;
  const int end = rp[i + 1];
  for (int kk = rp[i]; kk < diag[i]; ++kk) {
    const int k = ci[kk];
    double a[9], dk[9], l[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) { a[e] = v[(size_t)kk * 9 + e]; dk[e] = dinv[(size_t)k * 9 + e]; }
    mul3_exact(a, dk, l);
#pragma unroll
    for (int e = 0; e < 9; ++e) v[(size_t)kk * 9 + e] = l[e];
    int p = kk + 1;
    for (int jj = diag[k] + 1; jj < rp[k + 1]; ++jj) {
      const int j = ci[jj];
      while (p < end && ci[p] < j) ++p;
      if (p == end) break;
      if (ci[p] != j) continue;
      double u[9], t9[9];
#pragma unroll
      for (int e = 0; e < 9; ++e) u[e] = v[(size_t)jj * 9 + e];
      mul3_exact(l, u, t9);
#pragma unroll
      for (int e = 0; e < 9; ++e) v[(size_t)p * 9 + e] = dsub(v[(size_t)p * 9 + e], t9[e]);
    }
  }
  double dgl[9], inv[9];
#pragma unroll
  for (int e = 0; e < 9; ++e) dgl[e] = v[(size_t)diag[i] * 9 + e];
  if (!inv3_exact(dgl, inv)) {
    atomicMin(bad, i);
#pragma unroll
    for (int e = 0; e < 9; ++e) inv[e] = 0.0;
  }
#pragma unroll
  for (int e = 0; e < 9; ++e) dinv[(size_t)i * 9 + e] = inv[e];
}

// Sliced value array of one matrix from per-block values (9 doubles each),
// vsrc = source block per slot lane (-1: padding -> 0), optional transpose.
template <typename V>
__global__ void k_fill_sliced(long long slots, const int *__restrict__ vsrc, int transpose,
                              const double *__restrict__ src, V *__restrict__ out) {
  for (long long q = blockIdx.x * (long long)kThreads + threadIdx.x; q < slots * 32;
       q += (long long)gridDim.x * kThreads) {
    const long long slot = q >> 5;
    const int lane = (int)(q & 31);
    const int sblk = vsrc[q];
#pragma unroll
    for (int e = 0; e < 9; ++e) {
      const int ee = transpose ? (e % 3) * 3 + e / 3 : e;
      const double x = sblk >= 0 ? src[(size_t)sblk * 9 + ee] : 0.0;
      out[sl_idx<V>((size_t)slot, e, lane)] = (V)x;
    }
  }
}

// Sliced per-row 3x3 blocks (sl_idx, one slot per slice) from nb*9 doubles in
// permuted row order (drow: device row -> permuted row).
template <typename V>
__global__ void k_fill_diag(int S, const int2 *__restrict__ srows, const int *__restrict__ drow,
                            int transpose, const double *__restrict__ d, V *__restrict__ out) {
  for (long long q = blockIdx.x * (long long)kThreads + threadIdx.x; q < (long long)S * 32;
       q += (long long)gridDim.x * kThreads) {
    const int s = (int)(q >> 5), lane = (int)(q & 31);
    const int2 sr = srows[s];
#pragma unroll
    for (int e = 0; e < 9; ++e) {
      const int ee = transpose ? (e % 3) * 3 + e / 3 : e;
      const double x = lane < sr.y ? d[(size_t)drow[sr.x + lane] * 9 + ee] : 0.0;
      out[sl_idx<V>((size_t)s, e, lane)] = (V)x;
    }
  }
}

}  // namespace gbilu
