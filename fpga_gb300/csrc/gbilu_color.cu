// The parity-order greedy coloring (color_parity_greedy in gbilu_host.cpp)
// computed on the GPU, with the same result bit for bit. Every step of the
// host's sequential definition has an order-free parallel form:
//
//  1. face blocks: one thread per block row tests each of its blocks for a
//     4-cycle (the same predicate);
//  2. the lowest-numbered row of each connected part of the face graph:
//     minimum-label propagation with pointer jumping, to a fixed point;
//     breadth-first distances from those rows: one level per pass, a row
//     takes level L+1 when a face neighbour has level L (distances do not
//     depend on the visiting order);
//  3. moved rows: the host visits the equal-parity blocks (u, v), u < v, in
//     row-major order, and a block's decision reads only rows within one
//     block of u or v. A block is decided in the first pass in which every
//     earlier equal-parity block with an end within one block of u or v was
//     decided in an earlier pass; it then reads exactly what the host read
//     (passes are kernel launches, so those decisions are visible), and two
//     blocks decided in one pass never read each other's rows;
//  4. first-fit greedy in the order (parity 0, parity 1, moved; natural
//     order inside): a row is colored in the first pass in which all its
//     neighbours earlier in that order were colored in earlier passes
//     (Jones-Plassmann with the order as the priority), taking the smallest
//     color none of them holds -- what the host's sequential pass gives it.
//
// Used by gbilu_analyze when gbilu_options.color_on_device is set.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "gbilu_host.hpp"

namespace gbilu {
namespace {

constexpr int kT = 256;

__device__ __forceinline__ bool has_col(const int *ci, int b, int e, int x) {
  while (b < e) {   // binary search in a sorted column list
    const int m = (b + e) >> 1;
    const int c = ci[m];
    if (c == x) return true;
    if (c < x) b = m + 1; else e = m;
  }
  return false;
}

__device__ __forceinline__ int pos_of(const int *ci, int b, int e, int x) {
  while (b < e) {
    const int m = (b + e) >> 1;
    const int c = ci[m];
    if (c == x) return m;
    if (c < x) b = m + 1; else e = m;
  }
  return -1;
}

// 1. face[k] for every block of row u
__global__ void k_faces(int nb, const int *__restrict__ rp, const int *__restrict__ ci,
                        unsigned char *__restrict__ face) {
  for (int u = blockIdx.x * kT + threadIdx.x; u < nb; u += gridDim.x * kT) {
    const int ub = rp[u], ue = rp[u + 1];
    for (int k = ub; k < ue; ++k) {
      const int v = ci[k];
      bool found = false;
      if (v != u) {
        for (int kb = rp[v]; kb < rp[v + 1] && !found; ++kb) {
          const int b = ci[kb];
          if (b == v || b == u) continue;
          for (int ka = rp[b]; ka < rp[b + 1]; ++ka) {
            const int a = ci[ka];
            if (a != b && a != u && a != v && has_col(ci, ub, ue, a)) { found = true; break; }
          }
        }
      }
      face[k] = found;
    }
  }
}

// 2a. minimum label over face neighbours, then one pointer jump
__global__ void k_min_label(int nb, const int *__restrict__ rp, const int *__restrict__ ci,
                            const unsigned char *__restrict__ face, int *lab, int *changed) {
  for (int v = blockIdx.x * kT + threadIdx.x; v < nb; v += gridDim.x * kT) {
    int m = lab[v];
    for (int k = rp[v]; k < rp[v + 1]; ++k)
      if (face[k]) m = min(m, lab[ci[k]]);
    m = min(m, lab[m]);
    if (m < lab[v]) {
      lab[v] = m;
      *changed = 1;
    }
  }
}

__global__ void k_roots(int nb, const int *__restrict__ lab, int *dist) {
  for (int v = blockIdx.x * kT + threadIdx.x; v < nb; v += gridDim.x * kT)
    dist[v] = lab[v] == v ? 0 : -1;
}

// 2b. one breadth-first level: rows without a distance next to level L
__global__ void k_level(int nb, const int *__restrict__ rp, const int *__restrict__ ci,
                        const unsigned char *__restrict__ face, int L, int *dist, int *changed) {
  for (int v = blockIdx.x * kT + threadIdx.x; v < nb; v += gridDim.x * kT) {
    if (dist[v] >= 0) continue;
    for (int k = rp[v]; k < rp[v + 1]; ++k)
      if (face[k] && dist[ci[k]] == L) {
        dist[v] = L + 1;
        *changed = 1;
        break;
      }
  }
}

__device__ __forceinline__ bool same_parity(const int *dist, int a, int b) {
  return ((dist[a] ^ dist[b]) & 1) == 0;
}

// Whether any equal-parity block with an end in the closed neighbourhood of
// x and an index before key is still undecided (or was decided this pass).
__device__ bool earlier_open(const int *rp, const int *ci, const int *dist, const int *dround,
                             int x, int key, int pass) {
  for (int kx = rp[x]; kx < rp[x + 1]; ++kx) {
    const int y = ci[kx];
    if (y == x || !same_parity(dist, x, y)) continue;
    // the block (min, max) is kept at its index in the lower row
    const int kk = x < y ? kx : pos_of(ci, rp[y], rp[y + 1], x);
    if (kk < key && (dround[kk] == 0 || dround[kk] >= pass)) return true;
  }
  return false;
}

__device__ __forceinline__ bool touches_moved(const int *rp, const int *ci,
                                              const unsigned char *moved, int x) {
  for (int k = rp[x]; k < rp[x + 1]; ++k)
    if (moved[ci[k]]) return true;
  return false;
}

// 3. one pass over the undecided equal-parity blocks (u, v), u < v
__global__ void k_move_pass(int nb, const int *__restrict__ rp, const int *__restrict__ ci,
                            const int *__restrict__ dist, int *dround, unsigned char *moved,
                            int pass, int *open) {
  for (int u = blockIdx.x * kT + threadIdx.x; u < nb; u += gridDim.x * kT) {
    for (int k = rp[u]; k < rp[u + 1]; ++k) {
      const int v = ci[k];
      if (v <= u || !same_parity(dist, u, v) || dround[k] != 0) continue;
      bool ready = true;
      for (int t = rp[u]; t < rp[u + 1] && ready; ++t)
        if (earlier_open(rp, ci, dist, dround, ci[t], k, pass)) ready = false;
      for (int t = rp[v]; t < rp[v + 1] && ready; ++t)
        if (earlier_open(rp, ci, dist, dround, ci[t], k, pass)) ready = false;
      if (!ready) {
        *open = 1;
        continue;
      }
      if (!moved[u] && !moved[v]) {
        if (!touches_moved(rp, ci, moved, v)) moved[v] = 1;
        else if (!touches_moved(rp, ci, moved, u)) moved[u] = 1;
        else moved[v] = 1;
      }
      dround[k] = pass;
    }
  }
}

__device__ __forceinline__ long long order_key(const int *dist, const unsigned char *moved, int v) {
  const int cls = moved[v] ? 2 : (dist[v] & 1);
  return (long long)cls << 32 | (unsigned int)v;
}

// 4. one pass of first-fit greedy in the order key
__global__ void k_color_pass(int nb, const int *__restrict__ rp, const int *__restrict__ ci,
                             const int *__restrict__ dist, const unsigned char *__restrict__ moved,
                             int *cround, int *color, int pass, int *open) {
  for (int v = blockIdx.x * kT + threadIdx.x; v < nb; v += gridDim.x * kT) {
    if (cround[v] != 0) continue;
    const long long kv = order_key(dist, moved, v);
    bool ready = true;
    for (int k = rp[v]; k < rp[v + 1] && ready; ++k) {
      const int w = ci[k];
      if (w != v && order_key(dist, moved, w) < kv && (cround[w] == 0 || cround[w] >= pass))
        ready = false;
    }
    if (!ready) {
      *open = 1;
      continue;
    }
    // smallest color no earlier neighbour holds
    int c = 0;
    for (bool clash = true; clash; ) {
      clash = false;
      for (int k = rp[v]; k < rp[v + 1]; ++k) {
        const int w = ci[k];
        if (w != v && order_key(dist, moved, w) < kv && color[w] == c) {
          clash = true;
          ++c;
          break;
        }
      }
    }
    color[v] = c;
    cround[v] = pass;
  }
}

#define CKC(call)                                                              \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      err = std::string(#call ": ") + cudaGetErrorString(e_);                  \
      goto done;                                                               \
    }                                                                          \
  } while (0)

}  // namespace

std::string color_parity_device(int nb, const int *rowptr, const int *colind, int device,
                                int *color, int *ncolors, double *ms) {
  std::string err;
  const long long nnzb = rowptr[nb];
  int *d_rp = nullptr, *d_ci = nullptr, *d_lab = nullptr, *d_dist = nullptr, *d_dround = nullptr;
  int *d_cround = nullptr, *d_color = nullptr, *d_flag = nullptr;
  unsigned char *d_face = nullptr, *d_moved = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int sms = 0, h_flag = 0, grid = 0;
  std::vector<int> lab0;
  CKC(cudaSetDevice(device));
  CKC(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  grid = (int)std::min<long long>((nb + kT - 1) / kT, (long long)sms * 8);
  CKC(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  CKC(cudaEventCreate(&e0));
  CKC(cudaEventCreate(&e1));
  CKC(cudaMalloc(&d_rp, (nb + 1) * sizeof(int)));
  CKC(cudaMalloc(&d_ci, std::max<long long>(nnzb, 1) * sizeof(int)));
  CKC(cudaMalloc(&d_face, std::max<long long>(nnzb, 1)));
  CKC(cudaMalloc(&d_dround, std::max<long long>(nnzb, 1) * sizeof(int)));
  CKC(cudaMalloc(&d_lab, nb * sizeof(int)));
  CKC(cudaMalloc(&d_dist, nb * sizeof(int)));
  CKC(cudaMalloc(&d_cround, nb * sizeof(int)));
  CKC(cudaMalloc(&d_color, nb * sizeof(int)));
  CKC(cudaMalloc(&d_moved, nb));
  CKC(cudaMalloc(&d_flag, sizeof(int)));
  lab0.resize(nb);
  for (int i = 0; i < nb; ++i) lab0[i] = i;
  CKC(cudaEventRecord(e0, st));
  CKC(cudaMemcpyAsync(d_rp, rowptr, (nb + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
  CKC(cudaMemcpyAsync(d_ci, colind, nnzb * sizeof(int), cudaMemcpyHostToDevice, st));
  CKC(cudaMemcpyAsync(d_lab, lab0.data(), nb * sizeof(int), cudaMemcpyHostToDevice, st));
  CKC(cudaMemsetAsync(d_dround, 0, nnzb * sizeof(int), st));
  CKC(cudaMemsetAsync(d_cround, 0, nb * sizeof(int), st));
  CKC(cudaMemsetAsync(d_moved, 0, nb, st));
  k_faces<<<grid, kT, 0, st>>>(nb, d_rp, d_ci, d_face);
  // every loop below ends: each pass either changes something (a label
  // falls, a row gets a distance, a block or a row gets decided: the
  // earliest undecided one is always ready) or ends the loop, so nb + 2
  // passes (nnzb + 2 for the blocks) are more than any of them can take
  {
    const int kBatch = 16;   // passes between two looks at the flag
    for (int it = 0; it <= nb + 2; it += kBatch) {
      CKC(cudaMemsetAsync(d_flag, 0, sizeof(int), st));
      for (int j = 0; j < kBatch; ++j)
        k_min_label<<<grid, kT, 0, st>>>(nb, d_rp, d_ci, d_face, d_lab, d_flag);
      CKC(cudaMemcpyAsync(&h_flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
      CKC(cudaStreamSynchronize(st));
      if (!h_flag) break;
      if (it + kBatch > nb + 2) { err = "labels did not settle"; goto done; }
    }
    k_roots<<<grid, kT, 0, st>>>(nb, d_lab, d_dist);
    for (int L = 0; L <= nb + 2; L += kBatch) {
      CKC(cudaMemsetAsync(d_flag, 0, sizeof(int), st));
      for (int j = 0; j < kBatch; ++j)
        k_level<<<grid, kT, 0, st>>>(nb, d_rp, d_ci, d_face, L + j, d_dist, d_flag);
      CKC(cudaMemcpyAsync(&h_flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
      CKC(cudaStreamSynchronize(st));
      if (!h_flag) break;
    }
    for (long long pass = 1; pass <= nnzb + 2; ++pass) {
      CKC(cudaMemsetAsync(d_flag, 0, sizeof(int), st));
      k_move_pass<<<grid, kT, 0, st>>>(nb, d_rp, d_ci, d_dist, d_dround, d_moved, (int)pass,
                                       d_flag);
      CKC(cudaMemcpyAsync(&h_flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
      CKC(cudaStreamSynchronize(st));
      if (!h_flag) break;
      if (pass == nnzb + 2) { err = "moved rows did not settle"; goto done; }
    }
    for (int pass = 1; pass <= nb + 2; ++pass) {
      CKC(cudaMemsetAsync(d_flag, 0, sizeof(int), st));
      k_color_pass<<<grid, kT, 0, st>>>(nb, d_rp, d_ci, d_dist, d_moved, d_cround, d_color, pass,
                                        d_flag);
      CKC(cudaMemcpyAsync(&h_flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, st));
      CKC(cudaStreamSynchronize(st));
      if (!h_flag) break;
      if (pass == nb + 2) { err = "coloring did not settle"; goto done; }
    }
  }
  CKC(cudaMemcpyAsync(color, d_color, nb * sizeof(int), cudaMemcpyDeviceToHost, st));
  CKC(cudaEventRecord(e1, st));
  CKC(cudaStreamSynchronize(st));
  CKC(cudaGetLastError());
  {
    float t = 0.f;
    CKC(cudaEventElapsedTime(&t, e0, e1));
    if (ms) *ms = t;
  }
  {
    int mx = -1;
    for (int i = 0; i < nb; ++i) mx = std::max(mx, color[i]);
    *ncolors = mx + 1;
  }
done:
  for (void *p : {(void *)d_rp, (void *)d_ci, (void *)d_lab, (void *)d_dist, (void *)d_dround,
                  (void *)d_cround, (void *)d_color, (void *)d_flag, (void *)d_face,
                  (void *)d_moved})
    if (p) cudaFree(p);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  return err;
}

}  // namespace gbilu
