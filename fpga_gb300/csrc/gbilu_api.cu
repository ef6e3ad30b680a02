// C ABI of libgbilu.so (declared in include/gbilu.h): handle lifetime,
// device memory, the BiCGSTAB launch sequence, its CUDA graph (a device-side
// while loop), iterative refinement for the mixed mode and the adjoint.
#include "gbilu.h"
#include "gbilu_fpga_export.hpp"
#include "gbilu_host.hpp"
#include "gbilu_kernels.cuh"

#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

namespace gbilu {
namespace {

template <typename T> struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  cudaError_t alloc(size_t count) {
    n = count;
    return cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

// device copy of one sliced matrix
struct DevMat {
  DevBuf<int> off, col;
  DevBuf<int> vsrc;          // source block per slot lane (device factorization)
  bool transpose = false;
  long long slots = 0;
  DevBuf<double> v64;
  DevBuf<float> v32;
  void release() { off.release(); col.release(); vsrc.release(); v64.release(); v32.release(); }
};

// the work vectors of one BiCGSTAB run
template <typename T> struct Vecs {
  DevBuf<T> x, r, rt, p, ph, v, s, sh, t;
  DevBuf<T> y;               // first sweep of a preconditioner apply
  cudaError_t alloc(size_t n) {
    for (DevBuf<T> *b : {&x, &r, &rt, &p, &ph, &v, &s, &sh, &t, &y}) {
      cudaError_t e = b->alloc(n);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
  void release() {
    for (DevBuf<T> *b : {&x, &r, &rt, &p, &ph, &v, &s, &sh, &t, &y}) b->release();
  }
};

// Everything one BiCGSTAB run reads: operator, preconditioner and vectors.
template <typename V, typename T> struct Ops {
  bool transpose;
  const int *offA, *colA; const V *valA;     // A or A^T
  const int *off1, *col1; const V *val1;     // first sweep: L or U^T
  const int *off2, *col2; const V *val2;     // second sweep: U or L^T
  const V *dmat;                             // Dinv or Dinv^T (sliced)
  Vecs<T> *vec;
};

}  // namespace

struct Handle {
  gbilu_options opt{};
  std::string err;
  Analysis an;
  bool analyzed = false, factored = false;
  std::vector<double> pvals, lu, dinv;   // host: permuted A, factors
  double analyze_ms = 0, factor_ms = 0, color_ms = 0;
  // device
  bool dev_ready = false;
  int sm_count = 0;
  cudaStream_t st = nullptr, cap = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  // host-buffer solves move b on aux while the initial SpMV runs on st
  // (e_x: x0 is on the device; e_b: b is)
  cudaStream_t aux = nullptr;
  cudaEvent_t e_x = nullptr, e_b = nullptr;
  DevBuf<int2> srows;
  // perm/iperm: device row <-> input row (the vectors of a solve; lambda
  // of the gradient); dperm: device row -> permuted row (the device
  // factorization's layout); prowptr, pcol, psrc: the permuted pattern
  DevBuf<int> perm, iperm, dperm, prowptr, pcol, psrc;
  DevBuf<int> ibrow, icol;                   // input pattern: block -> row, column (dL/dA)
  DevMat A, L, U, At, Ut, Lt;
  DevBuf<double> dinv64, dinvT64;
  DevBuf<float> dinv32, dinvT32;
  Vecs<double> v64;
  Vecs<float> v32;
  DevBuf<double> b64, io64, io64b, partials, dA;
  DevBuf<int> x0nz;                        // set when x0 has a nonzero entry
  // device factorization: permuted values (factored in place), inverses
  DevBuf<int> pdiag, bad;
  DevBuf<double> pbuf, vals_in, dinvp;
  bool host_factors_stale = false;
  std::unique_ptr<FpgaExport> fpga;        // the last gbilu_fpga_export (sizes query)
  DevBuf<Ctl> ctl;                         // [0] main run, [1] refinement residual
  Ctl *h_ctl = nullptr;                    // pinned mirror
  bool with_t = false, with_32 = false;
  cudaGraphExec_t graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [fp32][transpose]
  cudaGraphExec_t graph_ru[2] = {nullptr, nullptr};  // mixed by replacement [transpose]
  int per_iter[2] = {0, 0};                // launches per iteration [transpose]
  long long last_launches = 0;
  // color steps [fp32][transpose]: the full list (one launch per step), and
  // the same as the single-launch apply's parameter when it fits (n = 0
  // otherwise: more than kMaxPhases / 2 colors)
  std::vector<Phase> steps[2][2];
  PhaseList phases[2][2];
  StagePlan stage[2][2] = {};              // shared-memory staging of small steps
  int stage_bytes[2][2] = {};
  DevBuf<StageEntry> stage_tab[2][2];
  DevBuf<int2> stage_cnt[2][2];
  DevBuf<unsigned int> ring_tab[2][2];     // streamed slices per CTA (see StagePlan)
  DevBuf<int> ring_cnt[2][2];
  cudaError_t launch_err = cudaSuccess;    // first failed cooperative launch
  int coop_grid64 = 1, coop_grid32 = 1;    // CTAs of the cooperative apply
  size_t device_bytes = 0;

  int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    err = buf;
    if (opt.verbose) printf("ERROR: %s\n", buf);
    return code;
  }
};

namespace {

#define CK(call)                                                                 \
  do {                                                                           \
    cudaError_t e_ = (call);                                                     \
    if (e_ != cudaSuccess)                                                       \
      return h->fail(GBILU_CUDA_ERROR, "%s: %s (%s:%d)", #call,                  \
                     cudaGetErrorString(e_), __FILE__, __LINE__);                \
  } while (0)

// the first launch error since the last check (cooperative launches report
// theirs through their return code)
cudaError_t last_error(Handle *h) {
  const cudaError_t e = cudaGetLastError();
  if (h->launch_err != cudaSuccess) {
    const cudaError_t le = h->launch_err;
    h->launch_err = cudaSuccess;
    return le;
  }
  return e;
}

int grid_for(const Handle *h, long long work) {
  long long g = (work + kThreads - 1) / kThreads;
  const long long cap = (long long)h->sm_count * 8;
  return (int)std::max<long long>(1, std::min(g, cap));
}

// Kernels that end in a grid reduction: fewer, fuller CTAs, so the
// last-CTA step sees few partials and few serialized arrival atomics.
#ifndef GBILU_REDUCE_CTAS_PER_SM
#define GBILU_REDUCE_CTAS_PER_SM 2
#endif
int reduce_grid(const Handle *h, long long work) {
  long long g = (work + kThreads - 1) / kThreads;
  const long long cap = (long long)h->sm_count * GBILU_REDUCE_CTAS_PER_SM;
  return (int)std::max<long long>(1, std::min(g, cap));
}

// ---------------------------------------------------------------------------
// launch sequences
// ---------------------------------------------------------------------------

// The color steps of one preconditioner apply, in execution order.
// Forward (z = U^-1 L^-1 src): the L sweep over colors 1..C-1 writes y for
// every row (color 0's y is src itself) and the final z = D^-1 y for the
// rows without a higher-colored neighbour; the U sweep then covers color 0
// and the leading rows of colors C-2..1. Transposed (z = L^-T U^-T src): the
// U^T sweep with D^-T over all colors, the rows without a higher-colored
// neighbour final at once (unit diagonal of L^T); the L^T sweep covers the
// leading rows of colors C-2..0.
std::vector<Phase> make_steps(const Analysis &an, bool transpose) {
  std::vector<Phase> st;
  const int C = an.ncolors;
  st.reserve(2 * (size_t)C);
  auto rows = [&](int c) { return an.color_ptr[c + 1] - an.color_ptr[c]; };
  auto add = [&](int c, int mat, int nrows) -> Phase & {
    st.emplace_back();
    Phase &p = st.back();
    p = Phase{};
    p.row0 = an.color_ptr[c];
    p.nrows = nrows;
    p.slice0 = an.slice_color_ptr[c];
    p.mat = mat;
    return p;
  };
  if (!transpose) {
    if (C == 1) {   // no couplings: z = D^-1 src
      add(0, 1, rows(0)).has_d = 1;
      return st;
    }
    for (int c = 1; c < C; ++c) {
      Phase &p = add(c, 0, rows(c));
      p.src_rows = an.color_ptr[1];
      p.to_y = 1;
      p.final0 = an.color_ptr[c] + an.split[c];
      p.final_d = 1;
    }
    for (int c = C - 2; c >= 0; --c) {
      const int nr = c == 0 ? rows(0) : an.split[c];
      if (nr == 0) continue;
      Phase &p = add(c, 1, nr);
      p.has_d = 1;
      p.own_y = c == 0 ? 0 : 1;
      p.nbr_hat = 1;
    }
  } else {
    for (int c = 0; c < C; ++c) {
      Phase &p = add(c, 0, rows(c));
      p.has_d = 1;
      p.to_y = 1;
      p.final0 = an.color_ptr[c] + an.split[c];
      p.final_d = 0;
    }
    for (int c = C - 2; c >= 0; --c) {
      if (an.split[c] == 0) continue;
      Phase &p = add(c, 1, an.split[c]);
      p.own_y = 1;
      p.nbr_hat = 1;
    }
  }
  // consecutive single-slice steps (the few rows of the top colors) run on
  // CTA 0, which orders them with a CTA barrier: one grid barrier less each;
  // consecutive small steps, once staged, need no barrier at all: they are
  // ordered by their data (sentinel polling in k_ilu_coop)
  for (size_t q = 0; q + 1 < st.size(); ++q) {
    st[q].local_after = st[q].nrows <= kSliceRows && st[q + 1].nrows <= kSliceRows;
    st[q].flow_after = st[q].nrows <= kSmallRows && st[q + 1].nrows <= kSmallRows;
  }
  return st;
}

// The single-launch apply's parameter (n = 0 when the steps do not fit).
PhaseList phase_list(const std::vector<Phase> &st) {
  PhaseList pl;
  pl.n = 0;
  pl.trace = 0;
  if (st.size() > (size_t)kMaxPhases) return pl;
  for (const Phase &p : st) pl.p[pl.n++] = p;
  return pl;
}

template <typename V, typename T>
int coop_grid(Handle *h) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ilu_coop<V, T>, coop_threads<T>(), 0);
  long long most = 0;
  for (int c = 0; c < h->an.ncolors; ++c) {
    const long long rows = h->an.color_ptr[c + 1] - h->an.color_ptr[c];
    most = std::max(most, rows);
  }
  const int need = (int)((most + coop_threads<T>() - 1) / coop_threads<T>());
  return std::max(1, std::min(per_sm * h->sm_count, need));
}

// Shared-memory staging of the small color steps (see StageEntry): slices are
// dealt round-robin to the CTAs of the cooperative grid; each CTA's entries
// pack [values | column indices | D^-1] at 128-byte multiples. Staging is
// off for this (precision, direction) when a CTA would need more than
// kStageBudget bytes or kMaxStage entries. The large steps' ring takes the
// shared memory left after the staged slices.
constexpr int kStageBudget = 160 * 1024;
// A ring of fewer stages than this leaves compute warps waiting for a
// stage (measured: the FP64 apply, 8 stages of 21.7 KB for 15 compute
// warps, 82 -> 118 us): no ring.
#ifndef GBILU_RING_MIN
#define GBILU_RING_MIN 12
#endif
constexpr int kRingMin = GBILU_RING_MIN;

// Bytes of one slice's [values | column indices | D block] in shared memory.
template <typename V>
long long slice_bytes(const SlicedMatrix &m, int slice, bool uses_d) {
  const long long w = m.off[slice + 1] - m.off[slice];
  return w * 9 * 32 * (long long)sizeof(V) + w * 32 * (long long)sizeof(int) +
         (uses_d ? 9 * 32 * (long long)sizeof(V) : 0);
}

template <typename V, typename T>
int build_stage_plan(Handle *h, int f, int t, int grid) {
  PhaseList &pl = h->phases[f][t];
  const Analysis &an = h->an;
  auto mat_of = [&](const Phase &P) -> const SlicedMatrix & {
    return t == 0 ? (P.mat ? an.U : an.L) : (P.mat ? an.Lt : an.Ut);
  };
  std::vector<std::vector<StageEntry>> per(grid);
  std::vector<long long> bytes(grid, 0);
  for (int q = 0; q < pl.n; ++q) {
    Phase &P = pl.p[q];
    P.staged = 0;
    P.streamed = 0;
    if (P.nrows > kSmallRows) continue;
    const SlicedMatrix &m = mat_of(P);
    const int nsl = (P.nrows + kSliceRows - 1) / kSliceRows;
    // steps linked by a CTA barrier (local_after) all run on CTA 0
    const bool local = P.local_after || (q > 0 && pl.p[q - 1].local_after);
    for (int j = 0; j < nsl; ++j) {
      const int b = local ? 0 : (j + q) % grid;
      per[b].push_back(StageEntry{q, j, m.off[P.slice0 + j + 1] - m.off[P.slice0 + j],
                                  (int)bytes[b]});
      bytes[b] += slice_bytes<V>(m, P.slice0 + j, P.uses_d());
    }
    P.staged = 1;
  }
  long long most = 0;
  size_t most_n = 0;
  for (int b = 0; b < grid; ++b) {
    most = std::max(most, bytes[b]);
    most_n = std::max(most_n, per[b].size());
  }
  h->stage[f][t] = StagePlan{nullptr, nullptr, 0, 0, 0, 0, nullptr, nullptr, 0};
  h->stage_bytes[f][t] = 0;
  const bool staged = h->opt.stage_small_steps && most_n > 0 && most <= kStageBudget &&
                      most_n <= (size_t)kMaxStage;
  if (!staged) {
    for (int q = 0; q < pl.n; ++q) pl.p[q].staged = 0;
    most = 0;
  }
  // the ring of the large (not staged) steps, after the staged slices
  int optin = 0;
  CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->opt.device));
  cudaFuncAttributes fa;
  CK(cudaFuncGetAttributes(&fa, k_ilu_coop<V, T>));
  const long long ring_off = (most + 127) / 128 * 128;
  long long stride = 0;
  bool any_large = false;
  // Only a large step that follows another step is streamed: its first
  // stages fill while the steps before it run. The first step of the
  // launch gains nothing from the ring (measured: FP32 L sweep of the
  // 500k-cell system 16.3 us from global memory, 21.2 us streamed).
  auto streamable = [&](int q) {
    const Phase &P = pl.p[q];
    return q > 0 && !P.staged && P.nrows > kSmallRows;
  };
  for (int q = 0; q < pl.n; ++q) {
    const Phase &P = pl.p[q];
    if (!streamable(q)) continue;
    any_large = true;
    const int nsl = (P.nrows + kSliceRows - 1) / kSliceRows;
    for (int j = 0; j < nsl; ++j)
      stride = std::max(stride, slice_bytes<V>(mat_of(P), P.slice0 + j, P.uses_d()));
  }
  stride = (stride + 127) / 128 * 128;
  const long long avail = (long long)optin - (long long)fa.sharedSizeBytes - ring_off;
// Stages of the FP32 ring: 12 is the best of 6..16 on the 500k-cell apply
// (a larger ring leaves less L1 for the large steps that read global
// memory: 8 stages 45.4 us, 12 41.9 us, 16 45.5 us)
#ifndef GBILU_RING_STAGES
#define GBILU_RING_STAGES 12
#endif
  const int ns = (stride > 0 && avail > 0)
                     ? (int)std::min<long long>(GBILU_RING_STAGES, avail / stride) : 0;
  const bool ring = h->opt.stream_large_steps && any_large && ns >= kRingMin;
  if (ring)
    for (int q = 0; q < pl.n; ++q) pl.p[q].streamed = streamable(q);
  const long long dyn = ring ? ring_off + ns * stride : most;
  if (dyn > 0) {
    CK(cudaFuncSetAttribute(k_ilu_coop<V, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)std::max<long long>(dyn, fa.maxDynamicSharedSizeBytes)));
    int per_sm = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ilu_coop<V, T>, coop_threads<T>(),
                                                     (size_t)dyn));
    if (per_sm < 1)
      return h->fail(GBILU_CUDA_ERROR, "single-launch apply does not fit an SM with %lld bytes "
                     "of shared memory", dyn);
  }
  StagePlan sp{nullptr, nullptr, 0, ring ? ns : 0, ring ? (int)stride : 0, (int)ring_off,
               nullptr, nullptr, 0};
  if (ring) {
    // each CTA's streamed slices in launch order: slice j of a step goes to
    // CTA j % grid
    std::vector<std::vector<unsigned int>> lists(grid);
    for (int q = 0; q < pl.n; ++q) {
      const Phase &P = pl.p[q];
      if (!P.streamed) continue;
      const int nsl = (P.nrows + kSliceRows - 1) / kSliceRows;
      for (int j = 0; j < nsl; ++j)
        lists[j % grid].push_back((unsigned int)(P.slice0 + j) | ((unsigned int)P.mat << 30) |
                                  ((unsigned int)P.uses_d() << 31));
    }
    size_t mx = 1;
    for (const auto &l : lists) mx = std::max(mx, l.size());
    std::vector<unsigned int> tab(mx * grid, 0u);
    std::vector<int> cnt(grid);
    for (int b = 0; b < grid; ++b) {
      std::copy(lists[b].begin(), lists[b].end(), tab.begin() + (size_t)b * mx);
      cnt[b] = (int)lists[b].size();
    }
    CK(h->ring_tab[f][t].alloc(tab.size()));
    CK(h->ring_cnt[f][t].alloc(cnt.size()));
    CK(cudaMemcpy(h->ring_tab[f][t].p, tab.data(), tab.size() * sizeof(unsigned int),
                  cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->ring_cnt[f][t].p, cnt.data(), cnt.size() * sizeof(int), cudaMemcpyHostToDevice));
    sp.ring_tab = h->ring_tab[f][t].p;
    sp.ring_cnt = h->ring_cnt[f][t].p;
    sp.ring_max = (int)mx;
  }
  if (staged) {
    std::vector<StageEntry> tab((size_t)grid * kMaxStage, StageEntry{0, 0, 0, 0});
    std::vector<int2> cnt(grid);
    for (int b = 0; b < grid; ++b) {
      for (size_t e = 0; e < per[b].size(); ++e) tab[(size_t)b * kMaxStage + e] = per[b][e];
      cnt[b] = make_int2((int)per[b].size(), (int)bytes[b]);
    }
    CK(h->stage_tab[f][t].alloc(tab.size()));
    CK(h->stage_cnt[f][t].alloc(cnt.size()));
    CK(cudaMemcpy(h->stage_tab[f][t].p, tab.data(), tab.size() * sizeof(StageEntry),
                  cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->stage_cnt[f][t].p, cnt.data(), cnt.size() * sizeof(int2),
                  cudaMemcpyHostToDevice));
    sp.tab = h->stage_tab[f][t].p;
    sp.cnt = h->stage_cnt[f][t].p;
    sp.enabled = 1;
  }
  h->stage[f][t] = sp;
  h->stage_bytes[f][t] = (int)dyn;
  return GBILU_OK;
}

// The single-launch preconditioner apply (cooperative, all CTAs resident).
template <typename V, typename T>
cudaError_t launch_coop(Handle *h, cudaStream_t s, const Ops<V, T> &o, const T *src, T *hat,
                        int trace) {
  const int f = sizeof(T) == 4 ? 1 : 0, t = o.transpose ? 1 : 0;
  PhaseList pl = h->phases[f][t];
  pl.trace = trace;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.gridDim = dim3(f ? h->coop_grid32 : h->coop_grid64);
  cfg.blockDim = dim3(coop_threads<T>());
  cfg.dynamicSmemBytes = (size_t)h->stage_bytes[f][t];
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_ilu_coop<V, T>, h->ctl.p, pl, h->stage[f][t], o.off1, o.col1,
                            o.val1, o.off2, o.col2, o.val2, o.dmat, src, o.vec->y.p, hat);
}

// hat = M^-1 src (forward) or M^-T src (transpose); the vector set's y holds
// the first sweep's result.
template <typename V, typename T>
void apply_prec(Handle *h, cudaStream_t s, const Ops<V, T> &o, const T *src, T *hat,
                int &launches) {
  const int C = h->an.ncolors;
  if (h->opt.sweep_mode == 1 && C <= kMaxPhases / 2) {
    const cudaError_t e = launch_coop(h, s, o, src, hat, 0);
    if (e != cudaSuccess && h->launch_err == cudaSuccess) h->launch_err = e;
    ++launches;
    return;
  }
  for (const Phase &P : h->steps[sizeof(T) == 4 ? 1 : 0][o.transpose ? 1 : 0]) {
    k_phase<V, T><<<(unsigned)((P.nrows + kThreads - 1) / kThreads), kThreads, 0, s>>>(
        h->ctl.p, P, P.mat ? o.off2 : o.off1, P.mat ? o.col2 : o.col1, P.mat ? o.val2 : o.val1,
        o.dmat, src, o.vec->y.p, hat);
    ++launches;
  }
}

template <typename V, typename T, int MODE>
void spmv(Handle *h, cudaStream_t s, const Ops<V, T> &o, const T *x, T *y, const T *w,
          int &launches, const int *x_nonzero = nullptr) {
  const int S = h->an.S;
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_spmv<V, T, MODE>, kThreads, 0);
  const int grid = std::max(1, std::min((S + kWarps - 1) / kWarps, std::max(1, per_sm) * h->sm_count));
  k_spmv<V, T, MODE><<<grid, kThreads, 0, s>>>(
      h->ctl.p, S, h->srows.p, o.offA, o.colA, o.valA, x, y, w, h->partials.p, x_nonzero);
  ++launches;
}

// One full BiCGSTAB iteration (both halves, PROGRAM steps 2-17).
// With ru64 (the FP64 operators; mixed precision by residual replacement)
// the iteration ends with the replacement kernels, which return at once
// unless a replacement is due.
template <typename V, typename T>
void enqueue_iteration(Handle *h, cudaStream_t s, const Ops<V, T> &o,
                       unsigned long long cond, int &launches,
                       const Ops<double, double> *ru64 = nullptr) {
  Vecs<T> &w = *o.vec;
  const int n = 3 * h->an.nb;
  const int g = grid_for(h, n);
  const int gr = reduce_grid(h, n);
  Ctl *c = h->ctl.p;
  double *part = h->partials.p;
  apply_prec(h, s, o, w.p.p, w.ph.p, launches);
  spmv<V, T, SPMV_ALPHA>(h, s, o, w.ph.p, w.v.p, w.rt.p, launches);
  k_update_s<T><<<gr, kThreads, 0, s>>>(c, n, w.r.p, w.v.p, w.s.p, part);
  apply_prec(h, s, o, w.s.p, w.sh.p, launches);
  spmv<V, T, SPMV_OMEGA>(h, s, o, w.sh.p, w.t.p, w.s.p, launches);
  k_update_r<T><<<gr, kThreads, 0, s>>>(c, n, w.x.p, w.ph.p, w.sh.p, w.s.p, w.t.p, w.rt.p,
                                        w.r.p, part);
  if (ru64 && sizeof(T) == 4) {
    Vecs<double> &d = h->v64;
    k_ru_accumulate<<<g, kThreads, 0, s>>>(c, n, (float *)w.x.p, d.x.p, 0);
    spmv<double, double, SPMV_TRUE>(h, s, *ru64, d.x.p, d.r.p, h->b64.p, launches);
    k_ru_replace<<<gr, kThreads, 0, s>>>(c, n, d.r.p, (float *)w.r.p, (const float *)w.rt.p, part);
    launches += 2;
  }
  k_update_p<T><<<g, kThreads, 0, s>>>(c, n, w.r.p, w.v.p, w.p.p, cond);
  launches += 3;
}

template <typename V, typename T>
int build_graph(Handle *h, const Ops<V, T> &o, cudaGraphExec_t &exec, int &per_iter,
                const Ops<double, double> *ru64 = nullptr) {
  cudaGraph_t g = nullptr;
  CK(cudaGraphCreate(&g, 0));
  cudaGraphConditionalHandle cond;
  CK(cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams params = {};
  params.type = cudaGraphNodeTypeConditional;
  params.conditional.handle = cond;
  params.conditional.type = cudaGraphCondTypeWhile;
  params.conditional.size = 1;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &params));
  cudaGraph_t body = params.conditional.phGraph_out[0];
  CK(cudaStreamBeginCaptureToGraph(h->cap, body, nullptr, nullptr, 0,
                                   cudaStreamCaptureModeThreadLocal));
  int launches = 0;
  enqueue_iteration(h, h->cap, o, (unsigned long long)cond, launches, ru64);
  cudaGraph_t captured = nullptr;
  CK(cudaStreamEndCapture(h->cap, &captured));
  CK(cudaGraphInstantiate(&exec, g, 0));
  CK(cudaGraphDestroy(g));
  per_iter = launches;
  return GBILU_OK;
}

template <typename V, typename T> Ops<V, T> make_ops(Handle *h, bool transpose);

template <> Ops<double, double> make_ops(Handle *h, bool t) {
  Ops<double, double> o;
  o.transpose = t;
  DevMat &a = t ? h->At : h->A, &m1 = t ? h->Ut : h->L, &m2 = t ? h->Lt : h->U;
  o.offA = a.off.p; o.colA = a.col.p; o.valA = a.v64.p;
  o.off1 = m1.off.p; o.col1 = m1.col.p; o.val1 = m1.v64.p;
  o.off2 = m2.off.p; o.col2 = m2.col.p; o.val2 = m2.v64.p;
  o.dmat = t ? h->dinvT64.p : h->dinv64.p;
  o.vec = &h->v64;
  return o;
}

template <> Ops<float, float> make_ops(Handle *h, bool t) {
  Ops<float, float> o;
  o.transpose = t;
  DevMat &a = t ? h->At : h->A, &m1 = t ? h->Ut : h->L, &m2 = t ? h->Lt : h->U;
  o.offA = a.off.p; o.colA = a.col.p; o.valA = a.v32.p;
  o.off1 = m1.off.p; o.col1 = m1.col.p; o.val1 = m1.v32.p;
  o.off2 = m2.off.p; o.col2 = m2.col.p; o.val2 = m2.v32.p;
  o.dmat = t ? h->dinvT32.p : h->dinv32.p;
  o.vec = &h->v32;
  return o;
}

// Runs the iteration loop of an already initialised Ctl (after the init
// kernels), as a graph or host-driven, then the x fix-up.
template <typename V, typename T>
int run_loop(Handle *h, bool transpose, int maxit, long long &launches, bool ru = false) {
  Ops<V, T> o = make_ops<V, T>(h, transpose);
  Ops<double, double> o64 = make_ops<double, double>(h, transpose);
  const Ops<double, double> *ru64 = ru ? &o64 : nullptr;
  const int fp32 = sizeof(T) == 4 ? 1 : 0, ti = transpose ? 1 : 0;
  const int n = 3 * h->an.nb;
  if (h->opt.use_graph) {
    cudaGraphExec_t &gx = ru ? h->graph_ru[ti] : h->graph[fp32][ti];
    if (!gx) {
      int rc = build_graph(h, o, gx, h->per_iter[ti], ru64);
      if (rc) return rc;
    }
    CK(cudaGraphLaunch(gx, h->st));
  } else {
    // host-driven: enqueue two iterations, then look at the done flag
    for (int it = 0; it <= maxit + 1; it += 2) {
      int l = 0;
      enqueue_iteration(h, h->st, o, 0ull, l, ru64);
      enqueue_iteration(h, h->st, o, 0ull, l, ru64);
      h->per_iter[ti] = l / 2;
      launches += l;
      CK(cudaMemcpyAsync(h->h_ctl, h->ctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost, h->st));
      CK(cudaStreamSynchronize(h->st));
      if (h->h_ctl->done) break;
    }
  }
  k_finish_x<T><<<grid_for(h, n), kThreads, 0, h->st>>>(h->ctl.p, n, o.vec->x.p, o.vec->ph.p);
  launches += 1;
  CK(last_error(h));
  return GBILU_OK;
}

void fill_result(const Handle *h, const Ctl &c, gbilu_result *res) {
  res->status = c.status;
  res->half_iters = c.status == ST_ALREADY || (c.status == ST_NONFINITE && c.half < 0) ? -1 : c.half;
  res->iterations = res->half_iters / 2.0 + 0.5;
  res->norm0 = c.norm0;
  res->norm = c.norm;
  res->relres = c.norm0 > 0 ? c.norm / c.norm0 : 0.0;
  for (int i = 0; i < 4; ++i) res->norms[i] = c.norms[i];
  res->last_norm_idx = c.last_norm_idx;
  (void)h;
}

// ---------------------------------------------------------------------------
// device set-up
// ---------------------------------------------------------------------------

int upload_mat(Handle *h, const SlicedMatrix &m, DevMat &d) {
  CK(d.off.alloc(m.off.size()));
  CK(d.col.alloc(m.col.size()));
  CK(cudaMemcpy(d.off.p, m.off.data(), m.off.size() * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d.col.p, m.col.data(), m.col.size() * sizeof(int), cudaMemcpyHostToDevice));
  const size_t nv = (size_t)m.slots() * 9 * kSliceRows;
  d.slots = m.slots();
  d.transpose = m.transpose_blocks;
  CK(d.v64.alloc(nv));
  if (h->with_32) CK(d.v32.alloc(nv));
  if (h->opt.factor_on_device) {
    CK(d.vsrc.alloc(m.vsrc.size()));
    CK(cudaMemcpy(d.vsrc.p, m.vsrc.data(), m.vsrc.size() * sizeof(int), cudaMemcpyHostToDevice));
    h->device_bytes += m.vsrc.size() * sizeof(int);
  }
  h->device_bytes += (m.off.size() + m.col.size()) * sizeof(int) + nv * 8 + (h->with_32 ? nv * 4 : 0);
  return GBILU_OK;
}

// A sliced value array of the host fill (FP64, entry-major: slots of
// [(slot*9 + e)*32 + l], which is the FP64 device layout) in the device
// layout of V (sl_idx); used for the FP32 copies.
template <typename V>
std::vector<V> to_device_layout(const std::vector<double> &em, size_t slots) {
  std::vector<V> out(em.size());
  for (size_t slot = 0; slot < slots; ++slot)
    for (int e = 0; e < 9; ++e)
      for (int l = 0; l < kSliceRows; ++l)
        out[sl_idx<V>(slot, e, l)] = (V)em[(slot * 9 + e) * kSliceRows + l];
  return out;
}

int upload_vals(Handle *h, const SlicedMatrix &m, const double *src, DevMat &d) {
  const size_t nv = (size_t)m.slots() * 9 * kSliceRows;
  std::vector<double> tmp(nv);
  fill_sliced<double>(m, src, tmp.data());   // the FP64 device layout already
  CK(cudaMemcpy(d.v64.p, tmp.data(), nv * sizeof(double), cudaMemcpyHostToDevice));
  if (h->with_32) {
    const std::vector<float> t32 = to_device_layout<float>(tmp, (size_t)m.slots());
    CK(cudaMemcpy(d.v32.p, t32.data(), nv * sizeof(float), cudaMemcpyHostToDevice));
  }
  return GBILU_OK;
}

int upload_diag(Handle *h, bool transpose, DevBuf<double> &d64, DevBuf<float> &d32) {
  const size_t nv = (size_t)h->an.S * 9 * kSliceRows;
  std::vector<double> tmp(nv);
  fill_sliced_diag<double>(h->an, h->dinv.data(), transpose, tmp.data());
  CK(cudaMemcpy(d64.p, tmp.data(), nv * sizeof(double), cudaMemcpyHostToDevice));
  if (h->with_32) {
    const std::vector<float> t32 = to_device_layout<float>(tmp, (size_t)h->an.S);
    CK(cudaMemcpy(d32.p, t32.data(), nv * sizeof(float), cudaMemcpyHostToDevice));
  }
  return GBILU_OK;
}

void release_device(Handle *h) {
  if (!h->dev_ready) return;
  cudaSetDevice(h->opt.device);
  for (auto &row : h->graph)
    for (auto &g : row)
      if (g) { cudaGraphExecDestroy(g); g = nullptr; }
  for (auto &g : h->graph_ru)
    if (g) { cudaGraphExecDestroy(g); g = nullptr; }
  for (DevMat *m : {&h->A, &h->L, &h->U, &h->At, &h->Ut, &h->Lt}) m->release();
  for (int f = 0; f < 2; ++f)
    for (int t = 0; t < 2; ++t) {
      h->stage_tab[f][t].release();
      h->stage_cnt[f][t].release();
      h->ring_tab[f][t].release();
      h->ring_cnt[f][t].release();
      h->stage[f][t] = StagePlan{nullptr, nullptr, 0, 0, 0, 0, nullptr, nullptr, 0};
      h->stage_bytes[f][t] = 0;
    }
  h->pdiag.release(); h->bad.release(); h->pbuf.release(); h->vals_in.release();
  h->dinvp.release();
  h->srows.release(); h->perm.release(); h->iperm.release(); h->dperm.release();
  h->ibrow.release(); h->icol.release();
  h->prowptr.release(); h->pcol.release();
  h->psrc.release(); h->dinv64.release(); h->dinvT64.release(); h->dinv32.release();
  h->dinvT32.release(); h->v64.release(); h->v32.release(); h->b64.release();
  h->io64.release(); h->io64b.release(); h->partials.release(); h->dA.release();
  h->x0nz.release();
  h->ctl.release();
  h->device_bytes = 0;
}

// Allocates the device side for the current analysis (structure only).
int setup_device(Handle *h) {
  if (h->opt.device < 0) return h->fail(GBILU_NO_DEVICE, "host-only handle has no device");
  CK(cudaSetDevice(h->opt.device));
  if (!h->st) {
    CK(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&h->cap, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&h->aux, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&h->e_x, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&h->e_b, cudaEventDisableTiming));
    CK(cudaEventCreate(&h->e0));
    CK(cudaEventCreate(&h->e1));
    CK(cudaMallocHost(&h->h_ctl, sizeof(Ctl)));
    CK(cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, h->opt.device));
  }
  release_device(h);
  h->dev_ready = true;
  const Analysis &an = h->an;
  const size_t n = 3 * (size_t)an.nb;
  h->with_t = true;
  h->with_32 = h->opt.precision == GBILU_MIXED;
  std::vector<int2> sr(an.S);
  for (int s = 0; s < an.S; ++s) sr[s] = make_int2(an.slice_row0[s], an.slice_len[s]);
  CK(h->srows.alloc(an.S));
  CK(cudaMemcpy(h->srows.p, sr.data(), sr.size() * sizeof(int2), cudaMemcpyHostToDevice));
  {
    std::vector<int> dv(an.nb), idv(an.nb);
    for (int d = 0; d < an.nb; ++d) {
      dv[d] = an.perm[an.dperm[d]];
      idv[dv[d]] = d;
    }
    CK(h->perm.alloc(an.nb));
    CK(cudaMemcpy(h->perm.p, dv.data(), an.nb * sizeof(int), cudaMemcpyHostToDevice));
    CK(h->iperm.alloc(an.nb));
    CK(cudaMemcpy(h->iperm.p, idv.data(), an.nb * sizeof(int), cudaMemcpyHostToDevice));
  }
  CK(h->dperm.alloc(an.nb));
  CK(cudaMemcpy(h->dperm.p, an.dperm.data(), an.nb * sizeof(int), cudaMemcpyHostToDevice));
  {
    std::vector<int> br(an.nnzb);
    for (int i = 0; i < an.nb; ++i)
      for (int k = an.rowptr[i]; k < an.rowptr[i + 1]; ++k) br[k] = i;
    CK(h->ibrow.alloc(an.nnzb));
    CK(cudaMemcpy(h->ibrow.p, br.data(), an.nnzb * sizeof(int), cudaMemcpyHostToDevice));
    CK(h->icol.alloc(an.nnzb));
    CK(cudaMemcpy(h->icol.p, an.colind.data(), an.nnzb * sizeof(int), cudaMemcpyHostToDevice));
  }
  CK(h->prowptr.alloc(an.nb + 1));
  CK(cudaMemcpy(h->prowptr.p, an.prowptr.data(), (an.nb + 1) * sizeof(int), cudaMemcpyHostToDevice));
  CK(h->pcol.alloc(an.nnzb));
  CK(cudaMemcpy(h->pcol.p, an.pcolind.data(), an.nnzb * sizeof(int), cudaMemcpyHostToDevice));
  CK(h->psrc.alloc(an.nnzb));
  CK(cudaMemcpy(h->psrc.p, an.psrc.data(), an.nnzb * sizeof(int), cudaMemcpyHostToDevice));
  for (auto pr : {std::make_pair(&an.A, &h->A), std::make_pair(&an.L, &h->L),
                  std::make_pair(&an.U, &h->U), std::make_pair(&an.At, &h->At),
                  std::make_pair(&an.Ut, &h->Ut), std::make_pair(&an.Lt, &h->Lt)}) {
    int rc = upload_mat(h, *pr.first, *pr.second);
    if (rc) return rc;
  }
  const size_t nd = (size_t)an.S * 9 * kSliceRows;
  CK(h->dinv64.alloc(nd));
  CK(h->dinvT64.alloc(nd));
  if (h->with_32) { CK(h->dinv32.alloc(nd)); CK(h->dinvT32.alloc(nd)); }
  CK(h->v64.alloc(n));
  if (h->with_32) CK(h->v32.alloc(n));
  CK(h->b64.alloc(n));
  CK(h->io64.alloc(n));
  CK(h->io64b.alloc(n));
  const size_t maxgrid = std::max<size_t>((size_t)h->sm_count * 8, (size_t)(an.S + kWarps - 1) / kWarps) + 1;
  CK(h->partials.alloc(2 * maxgrid));
  CK(h->x0nz.alloc(1));
  CK(cudaMemset(h->x0nz.p, 0xff, sizeof(int)));   // "nonzero" until a gather clears it
  CK(h->ctl.alloc(2));
  if (h->opt.factor_on_device) {
    CK(h->pdiag.alloc(an.nb));
    CK(cudaMemcpy(h->pdiag.p, an.pdiag.data(), an.nb * sizeof(int), cudaMemcpyHostToDevice));
    CK(h->bad.alloc(1));
    CK(h->pbuf.alloc((size_t)an.nnzb * 9));
    CK(h->vals_in.alloc((size_t)an.nnzb * 9));
    CK(h->dinvp.alloc((size_t)an.nb * 9));
    h->device_bytes += (size_t)an.nnzb * 9 * 16 + (size_t)an.nb * 76;
  }
  for (int f = 0; f < 2; ++f) {
    for (int t = 0; t < 2; ++t) {
      h->steps[f][t] = make_steps(an, t != 0);
      h->phases[f][t] = phase_list(h->steps[f][t]);
    }
  }
  h->coop_grid64 = coop_grid<double, double>(h);
  h->coop_grid32 = coop_grid<float, float>(h);
  if (an.ncolors <= kMaxPhases / 2) {
    for (int t = 0; t < 2; ++t) {
      int rc = build_stage_plan<double, double>(h, 0, t, h->coop_grid64);
      if (rc) return rc;
      if (h->with_32) {
        rc = build_stage_plan<float, float>(h, 1, t, h->coop_grid32);
        if (rc) return rc;
      }
    }
  }
  h->device_bytes += nd * 16 + (h->with_32 ? nd * 8 : 0) + n * 8 * 12 + (h->with_32 ? n * 4 * 9 : 0) +
                     (size_t)an.nnzb * 16 + (size_t)an.nb * 16;
  return GBILU_OK;
}

// Sliced values of one matrix (FP64 and, in the mixed mode, FP32) from
// per-block device values.
void fill_mat_device(Handle *h, DevMat &m, const double *src) {
  const int g = grid_for(h, m.slots * 32);
  k_fill_sliced<double><<<g, kThreads, 0, h->st>>>(m.slots, m.vsrc.p, m.transpose ? 1 : 0, src, m.v64.p);
  if (h->with_32)
    k_fill_sliced<float><<<g, kThreads, 0, h->st>>>(m.slots, m.vsrc.p, m.transpose ? 1 : 0, src, m.v32.p);
}

// Permute, factor and lay out on the device: values in input order (host
// array) -> color-permuted blocks -> A and A^T slices -> IKJ block ILU(0)
// color by color in place -> L, U, U^T, L^T and the inverse diagonal blocks.
int factor_device(Handle *h, const double *vals) {
  const Analysis &an = h->an;
  const size_t n9 = (size_t)an.nnzb * 9;
  CK(cudaMemcpyAsync(h->vals_in.p, vals, n9 * sizeof(double), cudaMemcpyHostToDevice, h->st));
  k_permute_blocks<<<grid_for(h, (long long)n9), kThreads, 0, h->st>>>(an.nnzb, h->psrc.p,
                                                                       h->vals_in.p, h->pbuf.p);
  fill_mat_device(h, h->A, h->pbuf.p);
  fill_mat_device(h, h->At, h->pbuf.p);
  const int big = 0x7fffffff;
  CK(cudaMemcpyAsync(h->bad.p, &big, sizeof(int), cudaMemcpyHostToDevice, h->st));
  for (int c = 0; c < an.ncolors; ++c) {
    const int row0 = an.color_ptr[c], rows = an.color_ptr[c + 1] - row0;
    k_bilu0_color<<<(rows + kThreads - 1) / kThreads, kThreads, 0, h->st>>>(
        row0, rows, h->prowptr.p, h->pcol.p, h->pdiag.p, h->pbuf.p, h->dinvp.p, h->bad.p);
  }
  int bad = big;
  CK(cudaMemcpyAsync(&bad, h->bad.p, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  CK(last_error(h));
  if (bad != big)
    return h->fail(GBILU_SINGULAR,
                   "gbilu_factor: singular diagonal block in permuted row %d (input row %d)", bad,
                   an.perm[bad]);
  fill_mat_device(h, h->L, h->pbuf.p);
  fill_mat_device(h, h->U, h->pbuf.p);
  fill_mat_device(h, h->Lt, h->pbuf.p);
  fill_mat_device(h, h->Ut, h->pbuf.p);
  const int gd = grid_for(h, (long long)an.S * 32);
  k_fill_diag<double><<<gd, kThreads, 0, h->st>>>(an.S, h->srows.p, h->dperm.p, 0, h->dinvp.p, h->dinv64.p);
  k_fill_diag<double><<<gd, kThreads, 0, h->st>>>(an.S, h->srows.p, h->dperm.p, 1, h->dinvp.p, h->dinvT64.p);
  if (h->with_32) {
    k_fill_diag<float><<<gd, kThreads, 0, h->st>>>(an.S, h->srows.p, h->dperm.p, 0, h->dinvp.p, h->dinv32.p);
    k_fill_diag<float><<<gd, kThreads, 0, h->st>>>(an.S, h->srows.p, h->dperm.p, 1, h->dinvp.p, h->dinvT32.p);
  }
  CK(cudaStreamSynchronize(h->st));
  CK(last_error(h));
  h->host_factors_stale = true;
  return GBILU_OK;
}

int check_solve_ready(Handle *h) {
  if (!h->analyzed) return h->fail(GBILU_NOT_READY, "gbilu_analyze has not been called");
  if (!h->factored) return h->fail(GBILU_NOT_READY, "gbilu_factor has not been called");
  if (h->opt.device < 0) return h->fail(GBILU_NO_DEVICE, "host-only handle cannot solve");
  return GBILU_OK;
}

// FP64 BiCGSTAB on the permuted vectors: b in h->b64, x in v64.x.
// With sync false the final Ctl is only queued for copy into h->h_ctl: the
// caller synchronizes once at the end (no host round trip mid-solve).
// b_ready: an event after which b is on the device (it is moved on another
// stream while A x0 is computed), or null when it is ready in stream order.
// b_in: b in the input numbering (permuted as it is read), or null for b64.
int solve64(Handle *h, bool transpose, double tol, int maxit, Ctl &out, long long &launches,
            bool sync = true, cudaEvent_t b_ready = nullptr, const double *b_in = nullptr) {
  const int n = 3 * h->an.nb;
  Ops<double, double> o = make_ops<double, double>(h, transpose);
  Vecs<double> &w = h->v64;
  const unsigned long long tmo = (unsigned long long)(h->opt.timeout_ms * 1e6);
  k_ctl_init<<<1, 32, 0, h->st>>>(h->ctl.p, tol, h->opt.absolute_tol, maxit, tmo);
  int l = 1;
  // r = A x0 (zeros without reading A when the gather of x0 found none)
  spmv<double, double, SPMV_PLAIN>(h, h->st, o, w.x.p, w.r.p, nullptr, l, h->x0nz.p);
  launches += l;
  if (b_ready) CK(cudaStreamWaitEvent(h->st, b_ready, 0));
  k_init_resid<double><<<reduce_grid(h, n), kThreads, 0, h->st>>>(
      h->ctl.p, n, b_in ? b_in : h->b64.p, b_in ? h->perm.p : nullptr, w.r.p, w.rt.p, w.p.p,
      h->partials.p);
  launches += 1;
  int rc = run_loop<double, double>(h, transpose, maxit, launches);
  if (rc) return rc;
  CK(cudaMemcpyAsync(h->h_ctl, h->ctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost, h->st));
  if (!sync) return GBILU_OK;
  CK(cudaStreamSynchronize(h->st));
  out = *h->h_ctl;
  if (h->opt.use_graph) launches += (long long)out.body_runs * h->per_iter[transpose ? 1 : 0];
  return GBILU_OK;
}

// Mixed precision by residual replacement: FP32 storage, sweeps and
// vectors, the FP32 correction accumulated into the FP64 x and the FP32
// residual replaced by the FP64 b - A x whenever the recursive residual fell
// by ru_delta (and when it reaches the bound); the stop is decided on the
// FP64 residual. The Krylov space is never restarted. b in h->b64, x in
// v64.x (FP64, permuted).
int solve_mixed_ru(Handle *h, bool transpose, double tol, int maxit, gbilu_result *res,
                   Ctl &out, long long &launches) {
  const int n = 3 * h->an.nb;
  Ops<double, double> o64 = make_ops<double, double>(h, transpose);
  Vecs<double> &w = h->v64;
  Vecs<float> &f = h->v32;
  const unsigned long long tmo = (unsigned long long)(h->opt.timeout_ms * 1e6);
  k_ctl_init<<<1, 32, 0, h->st>>>(h->ctl.p, tol, h->opt.absolute_tol, maxit, tmo);
  int l = 0;
  spmv<double, double, SPMV_RESID>(h, h->st, o64, w.x.p, w.r.p, h->b64.p, l);
  k_ru_init<<<reduce_grid(h, n), kThreads, 0, h->st>>>(h->ctl.p, n, h->opt.ru_delta, w.r.p, f.r.p,
                                                       f.rt.p, f.p.p, f.x.p, h->partials.p);
  launches += l + 2;
  int rc = run_loop<float, float>(h, transpose, maxit, launches, true);
  if (rc) return rc;
  // a stop after a first half owes xc += alpha p^ (k_finish_x in run_loop);
  // then the remaining FP32 correction goes into x
  k_ru_accumulate<<<grid_for(h, n), kThreads, 0, h->st>>>(h->ctl.p, n, f.x.p, w.x.p, 1);
  launches += 1;
  CK(cudaMemcpyAsync(h->h_ctl, h->ctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  out = *h->h_ctl;
  if (h->opt.use_graph) launches += (long long)out.body_runs * h->per_iter[transpose ? 1 : 0];
  if (out.status == ST_ALREADY || (out.status == ST_NONFINITE && out.half < 0)) return GBILU_OK;
  // report the FP64 residual of the returned x (recomputed unless the last
  // replacement just did)
  double tn = out.true_norm;
  if (out.status != ST_OK) {
    Ctl *outer = h->ctl.p + 1;
    k_ctl_init<<<1, 32, 0, h->st>>>(outer, 0.0, 1, 0, 0ull);
    const int S = h->an.S;
    k_spmv<double, double, SPMV_RESID><<<std::min((S + kWarps - 1) / kWarps, 2 * h->sm_count),
                                         kThreads, 0, h->st>>>(outer, S, h->srows.p, o64.offA,
                                                               o64.colA, o64.valA, w.x.p, w.r.p,
                                                               h->b64.p, h->partials.p);
    launches += 2;
    CK(cudaMemcpyAsync(h->h_ctl, outer, sizeof(Ctl), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    tn = h->h_ctl->norm0;
  }
  out.norm = tn;
  if (res) {
    res->outer_iters = out.replacements;
    res->inner_half_iters = out.half + 1;
    res->true_relres = out.norm0 > 0 ? tn / out.norm0 : 0.0;
  }
  return GBILU_OK;
}

// Mixed precision: FP32 inner BiCGSTAB inside FP64 iterative refinement.
// b in h->b64, x in v64.x (FP64, permuted).
int solve_mixed(Handle *h, bool transpose, double tol, int maxit, gbilu_result *res,
                Ctl &out, long long &launches) {
  if (h->opt.mixed_scheme == 1) return solve_mixed_ru(h, transpose, tol, maxit, res, out, launches);
  const int n = 3 * h->an.nb;
  Ops<double, double> o64 = make_ops<double, double>(h, transpose);
  Vecs<double> &w = h->v64;
  Vecs<float> &f = h->v32;
  Ctl *outer = h->ctl.p + 1;
  const int g = grid_for(h, n);
  auto residual = [&](double &nrm) -> int {
    // r = b - A x in FP64 with the FP64 copy of A, ||r|| read back
    k_ctl_init<<<1, 32, 0, h->st>>>(outer, 0.0, 1, 0, 0ull);
    const int S = h->an.S;
    k_spmv<double, double, SPMV_RESID><<<std::min((S + kWarps - 1) / kWarps, 2 * h->sm_count), kThreads, 0, h->st>>>(
        outer, S, h->srows.p, o64.offA, o64.colA, o64.valA, w.x.p, w.r.p, h->b64.p, h->partials.p);
    launches += 2;
    CK(cudaMemcpyAsync(h->h_ctl, outer, sizeof(Ctl), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    nrm = h->h_ctl->norm0;
    return GBILU_OK;
  };
  double nrm0 = 0, nrm = 0;
  int rc = residual(nrm0);
  if (rc) return rc;
  nrm = nrm0;
  memset(&out, 0, sizeof out);
  out.norm0 = nrm0;
  out.norms[0] = nrm0;
  out.status = ST_MAXIT;
  if (!std::isfinite(nrm0)) { out.status = ST_NONFINITE; out.half = -1; out.norm = nrm0; return GBILU_OK; }
  const double bound = h->opt.absolute_tol ? tol : tol * nrm0;
  if (!(nrm0 > (h->opt.absolute_tol ? tol : kAlreadySolved))) {
    out.status = ST_ALREADY; out.half = -1; out.norm = nrm0;
    return GBILU_OK;
  }
  const unsigned long long tmo = (unsigned long long)(h->opt.timeout_ms * 1e6);
  int outer_steps = 0, inner_half = 0;
  // maxit caps the inner half-iterations of all refinement steps together
  // the way the reference caps one run: at most maxit full iterations plus
  // the first half of one more, 2*maxit + 1 halves (solver.vhd:557). Each
  // inner solve gets the full iterations that still fit.
  const long long budget = 2LL * maxit + 1;
  while (nrm > bound && outer_steps < h->opt.max_outer && inner_half < budget) {
    const int left = (int)std::min<long long>((budget - inner_half - 1) / 2, h->opt.inner_maxit);
    // right-hand side of the correction equation A d = r / ||r|| in FP32
    // (staged in f.t, which the inner run overwrites only after reading it)
    k_scale_convert<<<g, kThreads, 0, h->st>>>(n, 1.0 / nrm, w.r.p, f.t.p);
    k_ctl_init<<<1, 32, 0, h->st>>>(h->ctl.p, h->opt.inner_tol, 0, left, tmo);
    k_init_rhs<float><<<reduce_grid(h, n), kThreads, 0, h->st>>>(h->ctl.p, n, f.t.p, f.r.p, f.rt.p,
                                                                 f.p.p, f.x.p, h->partials.p);
    launches += 3;
    rc = run_loop<float, float>(h, transpose, left, launches);
    if (rc) return rc;
    CK(cudaMemcpyAsync(h->h_ctl, h->ctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    const Ctl ic = *h->h_ctl;
    if (h->opt.use_graph) launches += (long long)ic.body_runs * h->per_iter[transpose ? 1 : 0];
    inner_half += (ic.half >= 0 ? ic.half + 1 : 0);
    ++outer_steps;
    if (ic.status == ST_BREAKDOWN || ic.status == ST_NONFINITE) { out.status = ic.status; break; }
    k_axpy_f2d<<<g, kThreads, 0, h->st>>>(n, nrm, f.x.p, w.x.p);
    launches += 1;
    rc = residual(nrm);
    if (rc) return rc;
    if (!std::isfinite(nrm)) { out.status = ST_NONFINITE; break; }
    if (ic.status == ST_TIMEOUT) { out.status = ST_TIMEOUT; break; }
  }
  if (nrm <= bound) out.status = ST_OK;
  out.norm = nrm;
  // the counter of one run that did all inner halves back to back
  out.half = inner_half - 1;
  if (res) {
    res->outer_iters = outer_steps;
    res->inner_half_iters = inner_half;
    res->true_relres = nrm0 > 0 ? nrm / nrm0 : 0.0;
  }
  out.norms[1] = nrm;
  out.last_norm_idx = 1;
  return GBILU_OK;
}

}  // namespace
}  // namespace gbilu

namespace gbilu {
namespace {
// One of the iteration's kernels for gbilu_bench_kernel (kind 4: SpMV with
// the alpha dot, 5: SpMV with the omega dots, 6-8: update_s/r/p).
template <typename V, typename T>
void iter_kernel(Handle *h, int kind, const Ops<V, T> &o, int n, int g, int gr, int &l) {
  Vecs<T> &w = *o.vec;
  if (kind == 4) {
    spmv<V, T, SPMV_ALPHA>(h, h->st, o, w.p.p, w.v.p, w.rt.p, l);
  } else if (kind == 5) {
    spmv<V, T, SPMV_OMEGA>(h, h->st, o, w.p.p, w.t.p, w.s.p, l);
  } else if (kind == 6) {
    k_update_s<T><<<gr, kThreads, 0, h->st>>>(h->ctl.p, n, w.r.p, w.v.p, w.s.p, h->partials.p);
    ++l;
  } else if (kind == 7) {
    k_update_r<T><<<gr, kThreads, 0, h->st>>>(h->ctl.p, n, w.x.p, w.ph.p, w.sh.p, w.s.p, w.t.p,
                                              w.rt.p, w.r.p, h->partials.p);
    ++l;
  } else {
    k_update_p<T><<<g, kThreads, 0, h->st>>>(h->ctl.p, n, w.r.p, w.v.p, w.p.p, 0ull);
    ++l;
  }
}
}  // namespace
}  // namespace gbilu

using namespace gbilu;

extern "C" {

int gbilu_default_options(gbilu_options *o) {
  if (!o) return GBILU_BAD_INPUT;
  memset(o, 0, sizeof *o);
  o->precision = GBILU_FP64;
  o->absolute_tol = 0;
  o->device = 0;
  o->use_graph = 1;
  o->timeout_ms = 0.0;
  o->inner_tol = 1e-1;
  o->inner_maxit = 500;
  o->max_outer = 30;
  o->verbose = 0;
  o->sweep_mode = 1;
  o->factor_on_device = 0;
  o->mixed_scheme = 0;
  o->ru_delta = 0.1;
  o->stage_small_steps = 1;
  o->coloring = 0;
  o->stream_large_steps = 0;
  o->color_on_device = 0;
  return GBILU_OK;
}

int gbilu_create(const gbilu_options *opt, void **handle) {
  if (!handle) return GBILU_BAD_INPUT;
  *handle = nullptr;
  Handle *h = new (std::nothrow) Handle();
  if (!h) return GBILU_BAD_INPUT;
  if (opt) h->opt = *opt; else gbilu_default_options(&h->opt);
  if (h->opt.precision != GBILU_FP64 && h->opt.precision != GBILU_MIXED) {
    delete h;
    return GBILU_BAD_INPUT;
  }
  *handle = h;
  return GBILU_OK;
}

int gbilu_destroy(void *handle) {
  Handle *h = static_cast<Handle *>(handle);
  if (!h) return GBILU_BAD_INPUT;
  if (h->st) {
    cudaSetDevice(h->opt.device);
    cudaStreamSynchronize(h->st);
    release_device(h);
    cudaStreamDestroy(h->st);
    cudaStreamDestroy(h->cap);
    cudaStreamDestroy(h->aux);
    cudaEventDestroy(h->e_x);
    cudaEventDestroy(h->e_b);
    cudaEventDestroy(h->e0);
    cudaEventDestroy(h->e1);
    cudaFreeHost(h->h_ctl);
  }
  delete h;
  return GBILU_OK;
}

int gbilu_analyze(void *handle, int nb, const int *rowptr, const int *colind) {
  Handle *h = static_cast<Handle *>(handle);
  if (!h) return GBILU_BAD_INPUT;
  auto t0 = std::chrono::steady_clock::now();
  h->analyzed = h->factored = false;
  h->fpga.reset();
  if (h->opt.coloring != 0 && h->opt.coloring != 1)
    return h->fail(GBILU_BAD_INPUT, "gbilu_analyze: coloring must be 0 or 1");
  std::vector<int> dcolors;
  h->color_ms = 0.0;
  if (h->opt.color_on_device && h->opt.device >= 0 && h->opt.coloring == 0) {
    // the pattern is checked first: the device coloring assumes it is valid
    std::string perr = check_pattern(nb, rowptr, colind);
    if (!perr.empty()) return h->fail(GBILU_BAD_INPUT, "gbilu_analyze: %s", perr.c_str());
    dcolors.resize(nb);
    int nc = 0;
    perr = color_parity_device(nb, rowptr, colind, h->opt.device, dcolors.data(), &nc, &h->color_ms);
    if (!perr.empty())
      return h->fail(GBILU_CUDA_ERROR, "gbilu_analyze: device coloring: %s", perr.c_str());
  }
  std::string err = analyze(nb, rowptr, colind, h->an, true, h->opt.coloring,
                            dcolors.empty() ? nullptr : dcolors.data(),
                            dcolors.empty() ? &h->color_ms : nullptr);
  if (!err.empty()) return h->fail(GBILU_BAD_INPUT, "gbilu_analyze: %s", err.c_str());
  h->analyzed = true;
  if (h->opt.device >= 0) {
    int rc = setup_device(h);
    if (rc) return rc;
  }
  h->analyze_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (h->opt.verbose)
    printf("INFO: gbilu_analyze: nb=%d nnzb=%d colors=%d slices=%d (%.1f ms)\n", nb, h->an.nnzb,
           h->an.ncolors, h->an.S, h->analyze_ms);
  return GBILU_OK;
}

int gbilu_get_ordering(void *handle, int *ncolors, int *color, int *perm, int *color_ptr) {
  Handle *h = static_cast<Handle *>(handle);
  if (!h) return GBILU_BAD_INPUT;
  if (!h->analyzed) return h->fail(GBILU_NOT_READY, "gbilu_analyze has not been called");
  if (ncolors) *ncolors = h->an.ncolors;
  if (color) memcpy(color, h->an.color.data(), h->an.nb * sizeof(int));
  if (perm) memcpy(perm, h->an.perm.data(), h->an.nb * sizeof(int));
  if (color_ptr) memcpy(color_ptr, h->an.color_ptr.data(), (h->an.ncolors + 1) * sizeof(int));
  return GBILU_OK;
}

int gbilu_factor(void *handle, const double *vals) {
  Handle *h = static_cast<Handle *>(handle);
  if (!h) return GBILU_BAD_INPUT;
  if (!h->analyzed) return h->fail(GBILU_NOT_READY, "gbilu_analyze has not been called");
  if (!vals) return h->fail(GBILU_BAD_INPUT, "vals must not be NULL");
  auto t0 = std::chrono::steady_clock::now();
  h->factored = false;
  h->fpga.reset();
  const Analysis &an = h->an;
  if (h->opt.factor_on_device && h->opt.device >= 0) {
    CK(cudaSetDevice(h->opt.device));
    h->pvals.clear();   // the host copies are only made when asked for
    const int rc = factor_device(h, vals);
    if (rc) return rc;
    h->factored = true;
    h->factor_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return GBILU_OK;
  }
  h->host_factors_stale = false;
  h->pvals.resize((size_t)an.nnzb * 9);
  permute_values(an, vals, h->pvals.data());
  h->lu = h->pvals;
  h->dinv.assign((size_t)an.nb * 9, 0.0);
  const int bad = bilu0(an, h->lu.data(), h->dinv.data());
  if (bad >= 0)
    return h->fail(GBILU_SINGULAR, "gbilu_factor: singular diagonal block in permuted row %d (input row %d)",
                   bad, an.perm[bad]);
  if (h->opt.device >= 0) {
    CK(cudaSetDevice(h->opt.device));
    int rc;
    if ((rc = upload_vals(h, an.A, h->pvals.data(), h->A))) return rc;
    if ((rc = upload_vals(h, an.L, h->lu.data(), h->L))) return rc;
    if ((rc = upload_vals(h, an.U, h->lu.data(), h->U))) return rc;
    if ((rc = upload_vals(h, an.At, h->pvals.data(), h->At))) return rc;
    if ((rc = upload_vals(h, an.Ut, h->lu.data(), h->Ut))) return rc;
    if ((rc = upload_vals(h, an.Lt, h->lu.data(), h->Lt))) return rc;
    if ((rc = upload_diag(h, false, h->dinv64, h->dinv32))) return rc;
    if ((rc = upload_diag(h, true, h->dinvT64, h->dinvT32))) return rc;
  }
  h->factored = true;
  h->factor_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return GBILU_OK;
}

int gbilu_get_factors(void *handle, double *lu, double *dinv) {
  Handle *h = static_cast<Handle *>(handle);
  if (!h) return GBILU_BAD_INPUT;
  if (!h->factored) return h->fail(GBILU_NOT_READY, "gbilu_factor has not been called");
  if (h->host_factors_stale) {      // factored on the device: fetch the copies
    CK(cudaSetDevice(h->opt.device));
    h->lu.resize((size_t)h->an.nnzb * 9);
    h->dinv.resize((size_t)h->an.nb * 9);
    CK(cudaMemcpy(h->lu.data(), h->pbuf.p, h->lu.size() * sizeof(double), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(h->dinv.data(), h->dinvp.p, h->dinv.size() * sizeof(double),
                  cudaMemcpyDeviceToHost));
    h->host_factors_stale = false;
  }
  if (lu) memcpy(lu, h->lu.data(), h->lu.size() * sizeof(double));
  if (dinv) memcpy(dinv, h->dinv.data(), h->dinv.size() * sizeof(double));
  return GBILU_OK;
}

int gbilu_fpga_export(void *handle, const double *b, const double *x0, int *vector_sizes,
                      int *nnz_sizes, void *const *vp) {
  Handle *h = static_cast<Handle *>(handle);
  if (!h) return GBILU_BAD_INPUT;
  if (!h->factored) return h->fail(GBILU_NOT_READY, "gbilu_factor has not been called");
  int rc = gbilu_get_factors(h, nullptr, nullptr);   // host copies of the factors
  if (rc) return rc;
  const Analysis &an = h->an;
  if (h->pvals.size() != (size_t)an.nnzb * 9) {
    // factored on the device: the permuted A from the uploaded input values
    std::vector<double> in((size_t)an.nnzb * 9);
    CK(cudaSetDevice(h->opt.device));
    CK(cudaMemcpy(in.data(), h->vals_in.p, in.size() * sizeof(double), cudaMemcpyDeviceToHost));
    h->pvals.resize(in.size());
    permute_values(an, in.data(), h->pvals.data());
  }
  if (!vp || !h->fpga) {
    auto ex = std::make_unique<FpgaExport>();
    const std::string err = fpga_export(an, h->pvals.data(), h->lu.data(), h->dinv.data(), *ex);
    if (!err.empty()) return h->fail(GBILU_BAD_INPUT, "gbilu_fpga_export: %s", err.c_str());
    h->fpga = std::move(ex);
  }
  const FpgaExport &ex = *h->fpga;
  if (vector_sizes) memcpy(vector_sizes, ex.vector_sizes, sizeof ex.vector_sizes);
  if (nnz_sizes) memcpy(nnz_sizes, ex.nnz_sizes, sizeof ex.nnz_sizes);
  if (!vp) return GBILU_OK;
  for (int m = 0; m < 3; ++m) {
    void *const *v = vp + 6 * m;
    if (!v[0] || !v[1] || !v[2] || !*(double *const *)v[2] || !v[3] || !v[4])
      return h->fail(GBILU_BAD_INPUT, "gbilu_fpga_export: a vector pointer is NULL");
    memcpy(v[0], ex.sizes[m].data(), ex.sizes[m].size() * sizeof(unsigned int));
    memcpy(v[1], ex.pidx[m].data(), ex.pidx[m].size() * sizeof(unsigned int));
    memcpy(*(double *const *)v[2], ex.vals[m].data(), ex.vals[m].size() * sizeof(double));
    memcpy(v[3], ex.cols[m].data(), ex.cols[m].size() * sizeof(unsigned short));
    memcpy(v[4], ex.nrs[m].data(), ex.nrs[m].size());
  }
  if (!vp[18] || !vp[19] || !vp[20])
    return h->fail(GBILU_BAD_INPUT, "gbilu_fpga_export: a vector pointer is NULL");
  memcpy(vp[18], ex.blkdiag.data(), ex.blkdiag.size() * sizeof(double));
  // rhs and x0 in the permuted numbering of the exported rows
  double *rhs = static_cast<double *>(vp[19]), *xx = static_cast<double *>(vp[20]);
  for (int i = 0; i < an.nb; ++i)
    for (int r = 0; r < 3; ++r) {
      rhs[3 * i + r] = b ? b[3 * (size_t)an.perm[i] + r] : 0.0;
      xx[3 * i + r] = x0 ? x0[3 * (size_t)an.perm[i] + r] : 0.0;
    }
  return GBILU_OK;
}

// One solve through the ABI. With gx and gdA (the adjoint), after the
// transposed solve the gradient dL/dA = -lambda_i x_j^T is formed on the
// device from lambda (still in the device vector) and gx (the forward
// solution, input numbering), inside the timed region, into gdA (input
// block order; host or device like the other arrays).
static int solve_impl(Handle *h, const double *b, double *x, bool device_ptrs, bool transpose,
                      double tol, int maxit, gbilu_result *res, const double *gx = nullptr,
                      double *gdA = nullptr) {
  int rc = check_solve_ready(h);
  if (rc) return rc;
  if (!b || !x) return h->fail(GBILU_BAD_INPUT, "b and x must not be NULL");
  if (maxit < 0) return h->fail(GBILU_BAD_INPUT, "maxit must be >= 0");
  if (!(tol >= 0.0)) return h->fail(GBILU_BAD_INPUT, "tol must be >= 0");
  auto t0 = std::chrono::steady_clock::now();
  CK(cudaSetDevice(h->opt.device));
  const int nb = h->an.nb, n = 3 * nb;
  const int g = grid_for(h, n);
  long long launches = 0;
  CK(cudaEventRecord(h->e0, h->st));
  const double *db = b;
  const double *dx = x;
  double *mapped_x = nullptr;
  if (!device_ptrs) {
    // Page-locked host buffers are read and written by the gather/scatter
    // kernels in place (mapped, over the CPU-GPU link); other host memory
    // goes through staging copies.
    cudaPointerAttributes ab, ax;
    const bool zb = cudaPointerGetAttributes(&ab, b) == cudaSuccess &&
                    ab.type == cudaMemoryTypeHost && ab.devicePointer;
    const bool zx = cudaPointerGetAttributes(&ax, x) == cudaSuccess &&
                    ax.type == cudaMemoryTypeHost && ax.devicePointer;
    cudaGetLastError();   // a query on unregistered memory is not an error here
    if (zb && zx) {
      db = static_cast<const double *>(ab.devicePointer);
      dx = mapped_x = static_cast<double *>(ax.devicePointer);
    } else {
      db = h->io64.p;   // staging copies below
      dx = h->io64b.p;
    }
  }
  // The FP64 solve needs b only after A x0 (k_init_resid): from host
  // buffers, b moves on the auxiliary stream while the SpMV runs. The
  // CPU-GPU link is one shared budget (about 200 GB/s for reads and writes
  // together, measured), so x0 goes first and alone; b follows on the copy
  // engine, which takes no SMs from the SpMV, and is permuted on the device.
  const bool fp64 = h->opt.precision != GBILU_MIXED;
  const bool overlap_b = fp64 && !device_ptrs;
  if (!device_ptrs && !mapped_x)
    CK(cudaMemcpyAsync(h->io64b.p, x, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
  CK(cudaMemsetAsync(h->x0nz.p, 0, sizeof(int), h->st));
  if (mapped_x)   // host side read in order, device side written permuted
    k_scatter<double><<<g, kThreads, 0, h->st>>>(nb, h->iperm.p, dx, h->v64.x.p, h->x0nz.p);
  else
    k_gather<double, double><<<g, kThreads, 0, h->st>>>(nb, h->perm.p, dx, h->v64.x.p, 1.0,
                                                        h->x0nz.p);
  cudaStream_t sb = h->st;
  if (overlap_b) {
    CK(cudaEventRecord(h->e_x, h->st));
    CK(cudaStreamWaitEvent(h->aux, h->e_x, 0));
    sb = h->aux;
  }
  if (!device_ptrs && (!mapped_x || overlap_b)) {
    CK(cudaMemcpyAsync(h->io64.p, b, n * sizeof(double), cudaMemcpyHostToDevice, sb));
    db = h->io64.p;
  }
  if (overlap_b)   // k_init_resid permutes b as it reads it
    CK(cudaEventRecord(h->e_b, h->aux));
  else if (mapped_x)
    k_scatter<double><<<g, kThreads, 0, sb>>>(nb, h->iperm.p, db, h->b64.p);
  else
    k_gather<double, double><<<g, kThreads, 0, sb>>>(nb, h->perm.p, db, h->b64.p, 1.0);
  launches += overlap_b ? 1 : 2;
  Ctl c;
  gbilu_result tmp;
  memset(&tmp, 0, sizeof tmp);
  gbilu_result *r = res ? res : &tmp;
  memset(r, 0, sizeof *r);
  if (!fp64)
    rc = solve_mixed(h, transpose, tol, maxit, r, c, launches);
  else
    rc = solve64(h, transpose, tol, maxit, c, launches, false, overlap_b ? h->e_b : nullptr,
                 overlap_b ? db : nullptr);
  if (rc) return rc;
  if (gx && gdA) {
    // lambda from the device numbering into the input numbering (x comes
    // in it), then dL/dA in the input block order
    const double *xin = gx;
    if (!device_ptrs) {   // b's staging buffer is free once the solve read it
      CK(cudaMemcpyAsync(h->io64.p, gx, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
      xin = h->io64.p;
    }
    k_scatter<double><<<g, kThreads, 0, h->st>>>(nb, h->perm.p, h->v64.x.p, h->v64.r.p);
    k_grad_a<<<grid_for(h, (long long)h->an.nnzb * 9), kThreads, 0, h->st>>>(
        h->an.nnzb, h->ibrow.p, h->icol.p, h->v64.r.p, xin, device_ptrs ? gdA : h->dA.p);
    launches += 2;
  }
  // x back to the caller's numbering. When the initial residual already met
  // the bound, v64.x still holds x0 (gathered), so this returns x0 unchanged
  // bit for bit; the FP64 path therefore needs no status before it and the
  // whole solve ends in one host synchronization.
  if (mapped_x)   // device side read permuted, host side written in order
    k_gather<double, double><<<g, kThreads, 0, h->st>>>(nb, h->iperm.p, h->v64.x.p, mapped_x, 1.0);
  else
    k_scatter<double><<<g, kThreads, 0, h->st>>>(nb, h->perm.p, h->v64.x.p,
                                                 device_ptrs ? x : h->io64b.p);
  launches += 1;
  CK(cudaEventRecord(h->e1, h->st));
  if (!device_ptrs && !mapped_x)
    CK(cudaMemcpyAsync(x, h->io64b.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  if (gx && gdA && !device_ptrs)
    CK(cudaMemcpyAsync(gdA, h->dA.p, (size_t)h->an.nnzb * 9 * sizeof(double),
                       cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  CK(last_error(h));
  if (fp64) {
    c = *h->h_ctl;
    if (h->opt.use_graph) launches += (long long)c.body_runs * h->per_iter[transpose ? 1 : 0];
  }
  const int outer = r->outer_iters, inner = r->inner_half_iters;
  const double tr = r->true_relres;
  fill_result(h, c, r);
  r->outer_iters = outer;
  r->inner_half_iters = inner;
  r->true_relres = h->opt.precision == GBILU_MIXED ? tr : r->relres;
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, h->e0, h->e1));
  r->device_ms = ms;
  r->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  h->last_launches = launches;
  if (h->opt.verbose)
    printf("INFO: gbilu_solve: status=%d half_iters=%d relres=%.3e device %.3f ms\n", r->status,
           r->half_iters, r->relres, r->device_ms);
  return GBILU_OK;
}

int gbilu_solve(void *handle, const double *b, double *x, double tol, int maxit, gbilu_result *res) {
  Handle *h = static_cast<Handle *>(handle);
  if (!h) return GBILU_BAD_INPUT;
  return solve_impl(h, b, x, false, false, tol, maxit, res);
}

int gbilu_solve_device(void *handle, const double *d_b, double *d_x, double tol, int maxit,
                       gbilu_result *res) {
  Handle *h = static_cast<Handle *>(handle);
  if (!h) return GBILU_BAD_INPUT;
  return solve_impl(h, d_b, d_x, true, false, tol, maxit, res);
}

int gbilu_apply_spmv(void *handle, const double *x, double *y, int transpose) {
  Handle *h = static_cast<Handle *>(handle);
  if (!h) return GBILU_BAD_INPUT;
  int rc = check_solve_ready(h);
  if (rc) return rc;
  if (!x || !y) return h->fail(GBILU_BAD_INPUT, "x and y must not be NULL");
  CK(cudaSetDevice(h->opt.device));
  const int nb = h->an.nb, n = 3 * nb, g = grid_for(h, n);
  Ops<double, double> o = make_ops<double, double>(h, transpose != 0);
  Vecs<double> &w = h->v64;
  int launches = 0;
  CK(cudaMemcpyAsync(h->io64.p, x, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
  k_gather<double, double><<<g, kThreads, 0, h->st>>>(nb, h->perm.p, h->io64.p, w.p.p, 1.0);
  spmv<double, double, SPMV_PLAIN>(h, h->st, o, w.p.p, w.v.p, nullptr, launches);
  k_scatter<double><<<g, kThreads, 0, h->st>>>(nb, h->perm.p, w.v.p, h->io64b.p);
  CK(cudaMemcpyAsync(y, h->io64b.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  CK(last_error(h));
  h->last_launches = launches + 2;
  return GBILU_OK;
}

int gbilu_apply_ilu(void *handle, const double *p, double *z, int transpose) {
  Handle *h = static_cast<Handle *>(handle);
  if (!h) return GBILU_BAD_INPUT;
  int rc = check_solve_ready(h);
  if (rc) return rc;
  if (!p || !z) return h->fail(GBILU_BAD_INPUT, "p and z must not be NULL");
  CK(cudaSetDevice(h->opt.device));
  const int nb = h->an.nb, n = 3 * nb, g = grid_for(h, n);
  const bool t = transpose != 0;
  Ops<double, double> o = make_ops<double, double>(h, t);
  Vecs<double> &w = h->v64;
  int launches = 0;
  k_ctl_init<<<1, 32, 0, h->st>>>(h->ctl.p, 0.0, 0, 0, 0ull);
  CK(cudaMemcpyAsync(h->io64.p, p, n * sizeof(double), cudaMemcpyHostToDevice, h->st));
  k_gather<double, double><<<g, kThreads, 0, h->st>>>(nb, h->perm.p, h->io64.p, w.p.p, 1.0);
  apply_prec(h, h->st, o, w.p.p, w.ph.p, launches);
  k_scatter<double><<<g, kThreads, 0, h->st>>>(nb, h->perm.p, w.ph.p, h->io64b.p);
  CK(cudaMemcpyAsync(z, h->io64b.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  CK(last_error(h));
  h->last_launches = launches + 3;
  return GBILU_OK;
}

int gbilu_adjoint(void *handle, const double *g_in, const double *x, double *lambda, double *dA,
                  double tol, int maxit, gbilu_result *res) {
  Handle *h = static_cast<Handle *>(handle);
  if (!h) return GBILU_BAD_INPUT;
  if (!g_in || !x || !lambda) return h->fail(GBILU_BAD_INPUT, "g, x and lambda must not be NULL");
  int rc = check_solve_ready(h);
  if (rc) return rc;
  if (dA && h->dA.n != (size_t)h->an.nnzb * 9) {
    CK(cudaSetDevice(h->opt.device));
    h->dA.release();
    CK(h->dA.alloc((size_t)h->an.nnzb * 9));
  }
  // lambda = A^-T g: the transposed solve, x0 = 0, then dL/dA on the device
  memset(lambda, 0, 3 * (size_t)h->an.nb * sizeof(double));
  return solve_impl(h, g_in, lambda, false, true, tol, maxit, res, dA ? x : nullptr, dA);
}

int gbilu_adjoint_device(void *handle, const double *d_g, const double *d_x, double *d_lambda,
                         double *d_dA, double tol, int maxit, gbilu_result *res) {
  Handle *h = static_cast<Handle *>(handle);
  if (!h) return GBILU_BAD_INPUT;
  if (!d_g || !d_x || !d_lambda)
    return h->fail(GBILU_BAD_INPUT, "g, x and lambda must not be NULL");
  int rc = check_solve_ready(h);
  if (rc) return rc;
  CK(cudaSetDevice(h->opt.device));
  CK(cudaMemsetAsync(d_lambda, 0, 3 * (size_t)h->an.nb * sizeof(double), h->st));
  return solve_impl(h, d_g, d_lambda, true, true, tol, maxit, res, d_dA ? d_x : nullptr, d_dA);
}

int gbilu_get_stats(void *handle, gbilu_stats *s) {
  Handle *h = static_cast<Handle *>(handle);
  if (!h || !s) return GBILU_BAD_INPUT;
  memset(s, 0, sizeof *s);
  if (!h->analyzed) return h->fail(GBILU_NOT_READY, "gbilu_analyze has not been called");
  const Analysis &an = h->an;
  s->nb = an.nb;
  s->nnzb = an.nnzb;
  s->ncolors = an.ncolors;
  s->nnzb_lower = an.nnzb_l;
  s->nnzb_upper = an.nnzb_u;
  s->slices = an.S;
  s->slots_a = an.A.slots();
  s->slots_l = an.L.slots();
  s->slots_u = an.U.slots();
  s->device_bytes = (long long)h->device_bytes;
  s->launches_per_iter = h->per_iter[0];
  s->last_launches = h->last_launches;
  s->factor_ms = h->factor_ms;
  s->analyze_ms = h->analyze_ms;
  s->color_ms = h->color_ms;
  s->color_on_device = h->opt.color_on_device && h->opt.device >= 0 && h->opt.coloring == 0;
  for (int p = 0; p < 2; ++p) {
    s->ring_stages[p] = h->stage[p][0].ring_ns;
    s->ring_stage_bytes[p] = h->stage[p][0].ring_stride;
    s->apply_smem_bytes[p] = h->stage_bytes[p][0];
  }
  for (int p = 0; p < 2; ++p) {
    const double sv = p ? 4.0 : 8.0, sx = sv, si = 4.0;
    const double nb = an.nb, n = 3.0 * an.nb;
    const double nlu = (double)an.nnzb_l + an.nnzb_u;
    s->alg_bytes_spmv[p] = an.nnzb * (9 * sv + si) + (nb + 1) * si + 2 * n * sx;
    s->alg_bytes_ilu[p] = nlu * (9 * sv + si) + 2 * (nb + 1) * si + nb * 9 * sv + 4 * n * sx;
    // fused vector kernels of one iteration: update_s (r, v -> s),
    // update_r (x, p^, s^, s, t, rt -> x, r), update_p (r, v, p -> p)
    // and the dot operands of the two SpMV epilogues (rt, s)
    const double vec = 17.0 * n * sx;
    s->alg_bytes_iter[p] = 2 * s->alg_bytes_spmv[p] + 2 * s->alg_bytes_ilu[p] + vec;
  }
  return GBILU_OK;
}

int gbilu_dot_check(void *handle, int n, const float *x, const float *y, double *dot_df,
                    double *dot_fp64) {
  Handle *h = static_cast<Handle *>(handle);
  if (!h || n <= 0 || !x || !y) return GBILU_BAD_INPUT;
  if (!h->analyzed) return h->fail(GBILU_NOT_READY, "gbilu_analyze has not been called");
  if (h->opt.device < 0) return h->fail(GBILU_NO_DEVICE, "host-only handle cannot run the check");
  if (!h->with_32) return h->fail(GBILU_BAD_INPUT, "the FP32 dot check needs GBILU_MIXED");
  if (n > 3 * h->an.nb) return h->fail(GBILU_BAD_INPUT, "n exceeds 3*nb");
  CK(cudaSetDevice(h->opt.device));
  Ctl *c = h->ctl.p + 1;   // the spare control block
  k_ctl_init<<<1, 32, 0, h->st>>>(c, 0.0, 0, 0, 0ull);
  CK(cudaMemcpyAsync(h->v32.r.p, x, n * sizeof(float), cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(h->v32.s.p, y, n * sizeof(float), cudaMemcpyHostToDevice, h->st));
  double out[2];
  for (int mode = 0; mode < 2; ++mode) {
    k_dot_check<<<reduce_grid(h, n), kThreads, 0, h->st>>>(c, n, h->v32.r.p, h->v32.s.p, mode,
                                                            h->partials.p);
    CK(cudaMemcpyAsync(h->h_ctl, c, sizeof(Ctl), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    out[mode] = h->h_ctl->dots[0];
  }
  CK(last_error(h));
  if (dot_df) *dot_df = out[0];
  if (dot_fp64) *dot_fp64 = out[1];
  return GBILU_OK;
}

int gbilu_wait_probe(void *handle, int mode, int *bar_fail, int *status, double *ms) {
  Handle *h = static_cast<Handle *>(handle);
  if (!h || (mode != 0 && mode != 1)) return GBILU_BAD_INPUT;
  if (!h->analyzed) return h->fail(GBILU_NOT_READY, "gbilu_analyze has not been called");
  if (h->opt.device < 0) return h->fail(GBILU_NO_DEVICE, "host-only handle cannot run the probe");
  CK(cudaSetDevice(h->opt.device));
  Ctl *c = h->ctl.p + 1;   // the spare control block: the solve state stays as it is
  k_ctl_init<<<1, 32, 0, h->st>>>(c, 0.0, 0, 0, 0ull);
  const unsigned long long sent = 0x7ff4a5a5a5a5a5a5ull;   // the data-ordered steps' sentinel
  CK(cudaMemcpyAsync(h->io64.p, &sent, sizeof sent, cudaMemcpyHostToDevice, h->st));
  CK(cudaEventRecord(h->e0, h->st));
  k_wait_probe<<<2, 32, 0, h->st>>>(c, mode, h->io64.p);
  CK(cudaEventRecord(h->e1, h->st));
  CK(cudaMemcpyAsync(h->h_ctl, c, sizeof(Ctl), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  CK(last_error(h));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, h->e0, h->e1));
  if (bar_fail) *bar_fail = h->h_ctl->bar_fail;
  if (status) *status = h->h_ctl->status;
  if (ms) *ms = t;
  return GBILU_OK;
}

int gbilu_device_order(void *handle, int *order) {
  Handle *h = static_cast<Handle *>(handle);
  if (!h || !order) return GBILU_BAD_INPUT;
  if (!h->analyzed) return h->fail(GBILU_NOT_READY, "gbilu_analyze has not been called");
  for (int d = 0; d < h->an.nb; ++d) order[d] = h->an.perm[h->an.dperm[d]];
  return GBILU_OK;
}

int gbilu_schedule(void *handle, int transpose, int cap, int *nsteps, int *steps) {
  Handle *h = static_cast<Handle *>(handle);
  if (!h) return GBILU_BAD_INPUT;
  if (!h->analyzed) return h->fail(GBILU_NOT_READY, "gbilu_analyze has not been called");
  const std::vector<Phase> st = make_steps(h->an, transpose != 0);
  if (nsteps) *nsteps = (int)st.size();
  for (int q = 0; q < (int)st.size() && q < cap && steps; ++q) {
    const Phase &P = st[q];
    // every step starts at a slice edge and ends with a grid barrier, a CTA
    // barrier when it and the next step run on CTA 0 alone, or none when
    // both are small (staged: the next step waits for the values it reads)
    const int v[13] = {P.row0, P.nrows, P.slice0, 0, P.mat, P.has_d, P.own_y, P.nbr_hat,
                       P.src_rows, P.to_y, P.final0, P.final_d,
                       P.flow_after ? 3 : P.local_after ? 2 : 1};
    memcpy(steps + 13 * q, v, sizeof v);
  }
  return GBILU_OK;
}

int gbilu_ilu_trace(void *handle, int fp32, int transpose, double *us, int *rows, int cap,
                    int *nphases) {
  Handle *h = static_cast<Handle *>(handle);
  if (!h) return GBILU_BAD_INPUT;
  int rc = check_solve_ready(h);
  if (rc) return rc;
  if (fp32 && !h->with_32) return h->fail(GBILU_BAD_INPUT, "FP32 trace needs GBILU_MIXED");
  if (h->an.ncolors > kMaxPhases / 2) return h->fail(GBILU_BAD_INPUT, "too many colors to trace");
  CK(cudaSetDevice(h->opt.device));
  const int t = transpose ? 1 : 0;
  const PhaseList &pl = h->phases[fp32 ? 1 : 0][t];
  const int n = 3 * h->an.nb;
  CK(cudaMemsetAsync(h->v64.p.p, 0, n * sizeof(double), h->st));
  if (h->with_32) CK(cudaMemsetAsync(h->v32.p.p, 0, n * sizeof(float), h->st));
  for (int rep = 0; rep < 2; ++rep) {   // the second, warm run is reported
    k_ctl_init<<<1, 32, 0, h->st>>>(h->ctl.p, 0.0, 0, 0, 0ull);
    if (fp32) {
      Ops<float, float> o = make_ops<float, float>(h, t != 0);
      CK(cudaMemsetAsync(h->v32.ph.p, 0, n * sizeof(float), h->st));
      CK(launch_coop(h, h->st, o, (const float *)h->v32.p.p, h->v32.ph.p, 1));
    } else {
      Ops<double, double> o = make_ops<double, double>(h, t != 0);
      CK(cudaMemsetAsync(h->v64.ph.p, 0, n * sizeof(double), h->st));
      CK(launch_coop(h, h->st, o, (const double *)h->v64.p.p, h->v64.ph.p, 1));
    }
  }
  CK(cudaMemcpyAsync(h->h_ctl, h->ctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  CK(last_error(h));
  if (nphases) *nphases = pl.n;
  for (int q = 0; q < pl.n && q < cap; ++q) {
    if (us) us[q] = (h->h_ctl->phase_ns[q + 1] - h->h_ctl->phase_ns[q]) * 1e-3;
    if (rows) rows[q] = pl.p[q].nrows;
  }
  return GBILU_OK;
}

int gbilu_bench_kernel(void *handle, int which, int reps, double *avg_ms, double *alg_bytes,
                       int *launches_out) {
  Handle *h = static_cast<Handle *>(handle);
  if (!h) return GBILU_BAD_INPUT;
  int rc = check_solve_ready(h);
  if (rc) return rc;
  if (which < 0 || which > 13 || reps <= 0) return h->fail(GBILU_BAD_INPUT, "bad kernel id or reps");
  const bool fp32 = which == 2 || which == 3 || which >= 9;
  if (fp32 && !h->with_32) return h->fail(GBILU_BAD_INPUT, "FP32 kernels need GBILU_MIXED");
  CK(cudaSetDevice(h->opt.device));
  gbilu_stats st;
  gbilu_get_stats(h, &st);
  const int nb = h->an.nb, n = 3 * nb, g = grid_for(h, n);
  int launches = 0;
  k_ctl_init<<<1, 32, 0, h->st>>>(h->ctl.p, 0.0, 0, 0, 0ull);
  // inputs: a fixed pseudo-random vector in the permuted numbering
  std::vector<double> x(n);
  uint64_t z = 0x9e3779b97f4a7c15ull;
  for (int i = 0; i < n; ++i) {
    z ^= z << 13; z ^= z >> 7; z ^= z << 17;
    x[i] = (double)(z >> 11) * (1.0 / 9007199254740992.0) - 0.5;
  }
  CK(cudaMemcpyAsync(h->v64.p.p, x.data(), n * sizeof(double), cudaMemcpyHostToDevice, h->st));
  if (h->with_32) k_scale_convert<<<g, kThreads, 0, h->st>>>(n, 1.0, h->v64.p.p, h->v32.p.p);
  if (which >= 4) {
    // every work vector of the iteration holds its own pseudo-random data,
    // so that the dots and norms are nonzero and no kernel stops the run
    Vecs<double> &w = h->v64;
    std::vector<double> xv(n);
    int k = 0;
    for (DevBuf<double> *b : {&w.x, &w.r, &w.rt, &w.ph, &w.v, &w.s, &w.sh, &w.t, &w.y}) {
      ++k;
      for (int i = 0; i < n; ++i) {
        z ^= z << 13; z ^= z >> 7; z ^= z << 17;
        xv[i] = ((double)(z >> 11) * (1.0 / 9007199254740992.0) - 0.5) * k;
      }
      CK(cudaMemcpyAsync(b->p, xv.data(), n * sizeof(double), cudaMemcpyHostToDevice, h->st));
      CK(cudaStreamSynchronize(h->st));
    }
    if (h->with_32) {
      Vecs<float> &f = h->v32;
      DevBuf<double> *src[9] = {&w.x, &w.r, &w.rt, &w.ph, &w.v, &w.s, &w.sh, &w.t, &w.y};
      DevBuf<float> *dst[9] = {&f.x, &f.r, &f.rt, &f.ph, &f.v, &f.s, &f.sh, &f.t, &f.y};
      for (int j = 0; j < 9; ++j)
        k_scale_convert<<<g, kThreads, 0, h->st>>>(n, 1.0, src[j]->p, dst[j]->p);
    }
  }
  // the iteration's other kernels (4-8 FP64, 9-13 FP32): the SpMV with the
  // alpha dot, the SpMV with the omega dots, update_s, update_r, update_p,
  // with solver scalars that never stop the run
  const int kind = which >= 9 ? which - 5 : which;
  if (which >= 4) k_ctl_bench<<<1, 32, 0, h->st>>>(h->ctl.p);
  const int gr = reduce_grid(h, n);
  auto run = [&](int &l) {
    if (which >= 9) {
      iter_kernel<float, float>(h, kind, make_ops<float, float>(h, false), n, g, gr, l);
    } else if (which >= 4) {
      iter_kernel<double, double>(h, kind, make_ops<double, double>(h, false), n, g, gr, l);
    } else if (which == 0) {
      Ops<double, double> o = make_ops<double, double>(h, false);
      spmv<double, double, SPMV_PLAIN>(h, h->st, o, h->v64.p.p, h->v64.v.p, nullptr, l);
    } else if (which == 1) {
      Ops<double, double> o = make_ops<double, double>(h, false);
      apply_prec(h, h->st, o, h->v64.p.p, h->v64.ph.p, l);
    } else if (which == 2) {
      Ops<float, float> o = make_ops<float, float>(h, false);
      spmv<float, float, SPMV_PLAIN>(h, h->st, o, h->v32.p.p, h->v32.v.p, nullptr, l);
    } else {
      Ops<float, float> o = make_ops<float, float>(h, false);
      apply_prec(h, h->st, o, h->v32.p.p, h->v32.ph.p, l);
    }
  };
  int warm = 0;
  for (int i = 0; i < 3; ++i) run(warm);
  CK(cudaStreamSynchronize(h->st));
  CK(cudaEventRecord(h->e0, h->st));
  for (int i = 0; i < reps; ++i) run(launches);
  CK(cudaEventRecord(h->e1, h->st));
  CK(cudaEventSynchronize(h->e1));
  CK(last_error(h));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, h->e0, h->e1));
  if (avg_ms) *avg_ms = ms / reps;
  if (alg_bytes) {
    const double sx = fp32 ? 4.0 : 8.0, nn = n;
    const int p = fp32 ? 1 : 0;
    // each operand read or written once: the SpMV plus its dot operand
    // (alpha: rt; omega: s), update_s r, v -> s; update_r x, p^, s^, s, t,
    // rt -> x, r; update_p r, v, p -> p
    const double by[5] = {st.alg_bytes_spmv[p] + nn * sx, st.alg_bytes_spmv[p] + nn * sx,
                          3 * nn * sx, 8 * nn * sx, 4 * nn * sx};
    *alg_bytes = which >= 4 ? by[kind - 4]
                            : (which == 0 || which == 2) ? st.alg_bytes_spmv[which / 2]
                                                         : st.alg_bytes_ilu[which / 2];
  }
  if (launches_out) *launches_out = launches / reps;
  return GBILU_OK;
}

const char *gbilu_status_string(int s) {
  switch (s) {
    case GBILU_OK: return "ok";
    case GBILU_MAXIT: return "maximum iterations reached";
    case GBILU_ALREADY_CONVERGED: return "initial residual already below the bound";
    case GBILU_BREAKDOWN: return "BiCGSTAB breakdown";
    case GBILU_NONFINITE: return "non-finite residual";
    case GBILU_TIMEOUT: return "device time budget exceeded";
    case GBILU_BAD_INPUT: return "bad input";
    case GBILU_SINGULAR: return "singular diagonal block";
    case GBILU_CUDA_ERROR: return "CUDA error";
    case GBILU_NOT_READY: return "call order";
    case GBILU_NO_DEVICE: return "host-only handle";
    default: return "unknown status";
  }
}

const char *gbilu_last_error(void *handle) {
  Handle *h = static_cast<Handle *>(handle);
  return h ? h->err.c_str() : "null handle";
}

}  // extern "C"
