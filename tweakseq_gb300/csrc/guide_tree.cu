// guide_tree.cu -- UPGMA / neighbour-joining guide trees from all-vs-all
// identities, on the GPU.
//
// This is the step the external multiple aligners run after their
// all-vs-all stage (the editor asks ClustalO for tree order,
// tweakseq/Core/ClustalO.cpp:51); the reference itself has no tree code, so
// the definition is the published methods (UPGMA: Sokal & Michener 1958;
// neighbour joining: Saitou & Nei 1987 in the Studier & Keppler 1988 form)
// over integer fixed-point distances (units of 2^-32).  Integers make every
// step exact: the result does not depend on summation order, and GB300's
// integer pipes are full rate where FP64 is not.
//
// Layout.  D is an n x n int64 matrix (row stride n) over *slots*: the m
// active clusters always occupy slots 0..m-1.  A join keeps the cluster at
// slot i and moves the last slot into slot j, so every scan reads a dense
// m x m upper triangle.  Each slot carries its canonical position (the
// position the textbook algorithm would give it: join t takes the smaller
// position of its children), so ties break exactly as in the position-
// ordered definition: smallest criterion, then smallest position pair.
//
// Two launches per join.  The scan: every block scans a share of the
// triangle (rows folded in pairs a, m-2-a so each share has m entries) and
// writes its best candidate; the last block to finish (atomic ticket, no
// waiting) picks and records the join.  The join: one thread per remaining
// slot updates the joined cluster's distances, the NJ row sums and the move
// of the last slot into the freed one.  The host issues the 2(n-1) launches
// with grids sized for the active count m = n - t, which it knows.
#include <climits>
#include <cstring>

#include "engine.h"

namespace tsq {
namespace {

constexpr int kTreeThreads = 256;

struct TreeState {
  int32_t m, t;
  uint32_t ticket;
  int32_t error;
  // The join the scan picked, for the join launch: slots i and j (pos[i] is
  // the smaller canonical position lo), the slot a the joined cluster takes
  // (i unless i is the last slot), the slot f that frees up, and the last
  // slot L that moves into f.
  int32_t i, j, a, f, L, lo, si, sj;
  int64_t dij;
};

struct Cand {
  int64_t c;
  int32_t lo, hi;  // canonical positions, lo < hi
  int32_t sa, sb;  // slots
};

__device__ __forceinline__ bool better(const Cand &x, const Cand &y) {
  if (x.c != y.c) return x.c < y.c;
  if (x.lo != y.lo) return x.lo < y.lo;
  return x.hi < y.hi;
}

__device__ __forceinline__ Cand shfl_cand(const Cand &x, int src) {
  Cand y;
  y.c = __shfl_sync(0xffffffffu, x.c, src);
  y.lo = __shfl_sync(0xffffffffu, x.lo, src);
  y.hi = __shfl_sync(0xffffffffu, x.hi, src);
  y.sa = __shfl_sync(0xffffffffu, x.sa, src);
  y.sb = __shfl_sync(0xffffffffu, x.sb, src);
  return y;
}

__device__ Cand block_best(Cand x, Cand *sm) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const Cand y = shfl_cand(x, (lane + o) & 31);
    if (better(y, x)) x = y;
  }
  if (lane == 0) sm[w] = x;
  __syncthreads();
  if (w == 0) {
    x = lane < kTreeThreads / 32 ? sm[lane] : sm[0];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const Cand y = shfl_cand(x, (lane + o) & 31);
      if (better(y, x)) x = y;
    }
    if (lane == 0) sm[0] = x;
  }
  __syncthreads();
  const Cand r = sm[0];
  __syncthreads();
  return r;
}

__device__ int64_t block_sum(int64_t v, int64_t *sm) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) sm[w] = v;
  __syncthreads();
  int64_t s = 0;
  for (int k = 0; k < kTreeThreads / 32; ++k) s += sm[k];
  __syncthreads();
  return s;
}

__device__ __forceinline__ int64_t floor_div(int64_t a, int64_t b) {
  int64_t q = a / b;
  if ((a % b != 0) && ((a < 0) != (b < 0))) --q;
  return q;
}

struct TreeArgs {
  int64_t *D;
  int64_t *r, *height;
  int32_t *pos, *node, *size;
  TreeState *st;
  Cand *partial;
  tsq_tree_node *out;
  int32_t n;
};

// Scan and pick: every block scans its share of the active triangle; the
// last block to finish (atomic ticket, no waiting) picks the join, records
// it and leaves the slots to the join launch.
template <bool NJ>
__global__ void __launch_bounds__(kTreeThreads) tree_scan_kernel(TreeArgs A, int32_t m, int32_t t) {
  __shared__ Cand sm_c[kTreeThreads / 32];
  __shared__ bool last;
  const int32_t n = A.n;
  if (m < 2 || A.st->error) return;
  const int64_t m2 = m - 2;

  Cand best{LLONG_MAX, INT_MAX, INT_MAX, -1, -1};
  const int32_t nfold = m / 2;
  for (int32_t fa = blockIdx.x; fa < nfold; fa += gridDim.x) {
    const int32_t a1 = fa, a2 = m - 2 - fa;
    const int32_t len1 = m - 1 - a1;
    const int32_t len2 = a2 != a1 ? m - 1 - a2 : 0;
    const int64_t r1 = NJ ? A.r[a1] : 0, r2 = NJ ? A.r[a2] : 0;
    const int32_t p1 = A.pos[a1], p2 = A.pos[a2];
    for (int32_t e = threadIdx.x; e < len1 + len2; e += kTreeThreads) {
      const bool first_row = e < len1;
      const int32_t row = first_row ? a1 : a2;
      const int32_t col = first_row ? a1 + 1 + e : a2 + 1 + (e - len1);
      const int64_t d = A.D[int64_t(row) * n + col];
      const int64_t c = NJ ? m2 * d - (first_row ? r1 : r2) - A.r[col] : d;
      if (c > best.c) continue;  // positions are only read for candidates that can win
      const int32_t pr = first_row ? p1 : p2, pc = A.pos[col];
      const Cand x{c, min(pr, pc), max(pr, pc), row, col};
      if (better(x, best)) best = x;
    }
  }
  best = block_best(best, sm_c);
  if (threadIdx.x == 0) {
    A.partial[blockIdx.x] = best;
    __threadfence();
    last = atomicAdd(&A.st->ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();

  best = Cand{LLONG_MAX, INT_MAX, INT_MAX, -1, -1};
  for (int k = threadIdx.x; k < int(gridDim.x); k += kTreeThreads) {
    const volatile Cand *vp = A.partial + k;
    const Cand x{vp->c, vp->lo, vp->hi, vp->sa, vp->sb};
    if (better(x, best)) best = x;
  }
  best = block_best(best, sm_c);
  if (threadIdx.x != 0) return;
  A.st->ticket = 0u;
  if (best.sa < 0) {
    A.st->error = 1;  // stops the remaining launches
    return;
  }
  const int32_t i = A.pos[best.sa] == best.lo ? best.sa : best.sb;
  const int32_t j = i == best.sa ? best.sb : best.sa;
  const int64_t dij = A.D[int64_t(i) * n + j];
  const int32_t si = A.size[i], sj = A.size[j];
  tsq_tree_node o;
  o.left = A.node[i];
  o.right = A.node[j];
  o.size = si + sj;
  o.pos = best.lo;
  o.dist = dij;
  if (NJ) {
    o.height = 0;
    o.left_length = m > 2 ? floor_div(m2 * dij + A.r[i] - A.r[j], 2 * m2) : (dij >> 1);
    o.right_length = dij - o.left_length;
  } else {
    const int64_t h = dij >> 1;
    o.height = h;
    o.left_length = h - A.height[i];
    o.right_length = h - A.height[j];
  }
  A.out[t] = o;
  const int32_t L = m - 1;
  const int32_t a = i != L ? i : j;
  A.st->i = i;
  A.st->j = j;
  A.st->a = a;
  A.st->f = a == i ? j : i;
  A.st->L = L;
  A.st->lo = best.lo;
  A.st->si = si;
  A.st->sj = sj;
  A.st->dij = dij;
  A.st->m = m - 1;  // for the host's final check only: the launches take m and t as arguments
  A.st->t = t + 1;
  if (NJ) A.r[a] = 0;  // the join launch adds the new row sum into it
}

// The join: one thread per remaining slot k.  Thread k writes the joined
// cluster's distance to k (row and column a) and, when the last slot L moves
// into the freed slot f, L's distance to k (row and column f); slot L's own
// thread writes the distance between the joined cluster and L at (a, f).
// Every thread touches only its own k's entries of rows/columns a and f and
// reads only rows i, j and L, so the updates are independent.
template <bool NJ>
__global__ void __launch_bounds__(kTreeThreads) tree_join_kernel(TreeArgs A, int32_t m, int32_t t) {
  __shared__ int64_t sm_s[kTreeThreads / 32];
  const TreeState st = *A.st;
  const int32_t n = A.n;
  if (m < 2 || st.error) return;
  const int32_t i = st.i, j = st.j, a = st.a, f = st.f, L = st.L;
  const int64_t dij = st.dij, si = st.si, sj = st.sj;
  const bool move = f != L;
  int64_t rsum = 0;
  for (int32_t k = blockIdx.x * kTreeThreads + threadIdx.x; k < m; k += gridDim.x * kTreeThreads) {
    if (k == i || k == j) continue;
    const int64_t dik = A.D[int64_t(i) * n + k], djk = A.D[int64_t(j) * n + k];
    const int64_t du = NJ ? (dik + djk - dij) >> 1 : floor_div(si * dik + sj * djk, si + sj);
    rsum += du;
    const int64_t rk = NJ ? A.r[k] + du - dik - djk : 0;
    if (move && k == L) {
      // L takes slot f.
      A.D[int64_t(a) * n + f] = du;
      A.D[int64_t(f) * n + a] = du;
      A.D[int64_t(f) * n + f] = 0;
      if (NJ) A.r[f] = rk;
      A.height[f] = A.height[L];
      A.pos[f] = A.pos[L];
      A.node[f] = A.node[L];
      A.size[f] = A.size[L];
    } else {
      A.D[int64_t(a) * n + k] = du;
      A.D[int64_t(k) * n + a] = du;
      if (NJ) A.r[k] = rk;
      if (move) {
        const int64_t dlk = A.D[int64_t(L) * n + k];
        A.D[int64_t(f) * n + k] = dlk;
        A.D[int64_t(k) * n + f] = dlk;
      }
    }
  }
  if (NJ) {
    rsum = block_sum(rsum, sm_s);
    if (threadIdx.x == 0 && rsum != 0) atomicAdd(reinterpret_cast<unsigned long long *>(A.r + a),
                                                 static_cast<unsigned long long>(rsum));
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (!NJ) A.height[a] = dij >> 1;
    A.node[a] = n + t;
    A.size[a] = int32_t(si + sj);
    A.pos[a] = st.lo;
    A.D[int64_t(a) * n + a] = 0;
  }
}

__device__ __forceinline__ int64_t identity_distance(int32_t n_ident, int32_t n_cols) {
  if (n_cols <= 0) return int64_t(1) << 32;
  return int64_t((uint64_t(uint32_t(n_cols - n_ident)) << 32) / uint64_t(uint32_t(n_cols)));
}

// D from identities of the unordered pairs (i < j) in row-major order; the
// identities sit `stride` int32 apart (1 for plain arrays, 8 for ResultDev
// records), with the pair status `status_off` ints after n_ident (or none).
__global__ void tree_init_kernel(int64_t *D, int32_t n, const int32_t *ident, const int32_t *cols, int32_t stride,
                                 const int32_t *status, TreeState *st) {
  const int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  const int32_t i = blockIdx.y;
  if (j >= n) return;
  if (i == j) {
    D[int64_t(i) * n + j] = 0;
    return;
  }
  const int32_t lo = min(i, j), hi = max(i, j);
  const int64_t k = int64_t(lo) * (2 * int64_t(n) - lo - 1) / 2 + (hi - lo - 1);
  const int32_t ni = ident[k * stride], nc = cols[k * stride];
  if ((status && status[k * stride] != 0) || nc < 0 || ni < 0 || ni > nc) st->error = 2;
  D[int64_t(i) * n + j] = identity_distance(ni, nc);
}

__global__ void tree_slots_kernel(const int64_t *D, int32_t n, int64_t *r, int64_t *height, int32_t *pos,
                                  int32_t *node, int32_t *size, TreeState *st) {
  const int32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w == 0 && lane == 0) {
    st->m = n;
    st->t = 0;
    st->ticket = 0u;
  }
  if (w >= n) return;
  int64_t s = 0;
  for (int32_t k = lane; k < n; k += 32)
    if (k != w) s += D[int64_t(w) * n + k];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) {
    r[w] = s;
    height[w] = 0;
    pos[w] = w;
    node[w] = w;
    size[w] = 1;
  }
}

__global__ void tree_error_reset_kernel(TreeState *st) { st->error = 0; }

int sm_count() {
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

struct TreeBufs {
  DevBuf D, small, partial, out;
  cudaStream_t stream = nullptr;
  int dev = -1;
  ~TreeBufs() {
    if (stream) cudaStreamDestroy(stream);
  }
};

constexpr int32_t kMaxTreeLeaves = 65535;  // one grid row per leaf in tree_init_kernel

// Sizes the buffers for n leaves and fills TreeArgs.
cudaError_t tree_prepare(TreeBufs &b, int32_t n, TreeArgs *A) {
  const size_t nn = size_t(n) * size_t(n);
  cudaError_t e = b.D.ensure(nn * 8);
  const size_t small = size_t(n) * (8 + 8 + 4 + 4 + 4) + sizeof(TreeState) + 64;
  if (e == cudaSuccess) e = b.small.ensure(small);
  const int parts = 4 * sm_count();
  if (e == cudaSuccess) e = b.partial.ensure(size_t(parts) * sizeof(Cand));
  if (e == cudaSuccess) e = b.out.ensure(size_t(n > 1 ? n - 1 : 1) * sizeof(tsq_tree_node));
  if (e != cudaSuccess) return e;
  char *p = b.small.as<char>();
  A->D = b.D.as<int64_t>();
  A->r = reinterpret_cast<int64_t *>(p);
  A->height = A->r + n;
  A->pos = reinterpret_cast<int32_t *>(A->height + n);
  A->node = A->pos + n;
  A->size = A->node + n;
  A->st = reinterpret_cast<TreeState *>((reinterpret_cast<uintptr_t>(A->size + n) + 15) & ~uintptr_t(15));
  A->partial = b.partial.as<Cand>();
  A->out = b.out.as<tsq_tree_node>();
  A->n = n;
  return cudaSuccess;
}

// Row sums, slot tables, then the n-1 joins; copies the joins to `out`.
int tree_run(const TreeArgs &A, int32_t method, cudaStream_t s, tsq_tree_node *out) {
  const int32_t n = A.n;
  tree_slots_kernel<<<(n + 7) / 8, 256, 0, s>>>(A.D, n, A.r, A.height, A.pos, A.node, A.size, A.st);
  const int parts = 4 * sm_count();
  for (int32_t t = 0; t < n - 1; ++t) {
    const int32_t m = n - t;
    const int blocks = std::max(1, std::min(parts, m / 2));
    const int jblocks = std::max(1, std::min(parts, (m + kTreeThreads - 1) / kTreeThreads));
    if (method == TSQ_TREE_NJ) {
      tree_scan_kernel<true><<<blocks, kTreeThreads, 0, s>>>(A, m, t);
      tree_join_kernel<true><<<jblocks, kTreeThreads, 0, s>>>(A, m, t);
    } else {
      tree_scan_kernel<false><<<blocks, kTreeThreads, 0, s>>>(A, m, t);
      tree_join_kernel<false><<<jblocks, kTreeThreads, 0, s>>>(A, m, t);
    }
  }
  cudaError_t e = cudaGetLastError();
  TreeState st{};
  if (e == cudaSuccess) e = cudaMemcpyAsync(&st, A.st, sizeof(st), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && n > 1)
    e = cudaMemcpyAsync(out, A.out, sizeof(tsq_tree_node) * size_t(n - 1), cudaMemcpyDeviceToHost, s);
  const cudaError_t sy = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = sy;
  if (e != cudaSuccess) return cuda_status(e);
  if (st.error == 2) return TSQ_E_INVALID_ARG;
  if (st.error != 0 || st.m != 1 || st.t != n - 1) return TSQ_E_CUDA;
  return TSQ_OK;
}

TreeBufs &tree_cache(int *rc) {
  thread_local TreeBufs c;
  int dev = 0;
  *rc = TSQ_OK;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    *rc = TSQ_E_CUDA;
    return c;
  }
  if (c.dev != dev) {
    c.D.release();
    c.small.release();
    c.partial.release();
    c.out.release();
    if (c.stream) cudaStreamDestroy(c.stream);
    c.stream = nullptr;
    if (cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess) {
      *rc = TSQ_E_CUDA;
      return c;
    }
    c.dev = dev;
  }
  return c;
}

bool bad_method(int32_t method) { return method != TSQ_TREE_UPGMA && method != TSQ_TREE_NJ; }

}  // namespace
}  // namespace tsq

extern "C" {

int tsq_guide_tree_dist(int32_t n, const int64_t *dist, int32_t method, tsq_tree_node *out) {
  if (n < 1 || n > tsq::kMaxTreeLeaves || !dist || tsq::bad_method(method) || (n > 1 && !out))
    return TSQ_E_INVALID_ARG;
  if (n == 1) return TSQ_OK;
  for (int32_t i = 0; i < n; ++i)
    for (int32_t j = i + 1; j < n; ++j)
      if (dist[int64_t(i) * n + j] != dist[int64_t(j) * n + i]) return TSQ_E_INVALID_ARG;
  try {
    int rc = TSQ_OK;
    tsq::TreeBufs &b = tsq::tree_cache(&rc);
    if (rc) return rc;
    tsq::TreeArgs A;
    cudaError_t e = tsq::tree_prepare(b, n, &A);
    if (e == cudaSuccess) e = cudaMemcpyAsync(A.D, dist, size_t(n) * size_t(n) * 8, cudaMemcpyHostToDevice, b.stream);
    if (e == cudaSuccess) {
      tsq::tree_error_reset_kernel<<<1, 1, 0, b.stream>>>(A.st);
      e = cudaGetLastError();
    }
    if (e != cudaSuccess) return tsq::cuda_status(e);
    return tsq::tree_run(A, method, b.stream, out);
  } catch (const std::bad_alloc &) {
    return TSQ_E_NOMEM;
  }
}

int tsq_guide_tree(int32_t n, const int32_t *n_ident, const int32_t *n_cols, int32_t method, tsq_tree_node *out) {
  if (n < 1 || n > tsq::kMaxTreeLeaves || tsq::bad_method(method) || (n > 1 && (!out || !n_ident || !n_cols)))
    return TSQ_E_INVALID_ARG;
  if (n == 1) return TSQ_OK;
  try {
    int rc = TSQ_OK;
    tsq::TreeBufs &b = tsq::tree_cache(&rc);
    if (rc) return rc;
    tsq::TreeArgs A;
    const int64_t npairs = int64_t(n) * (n - 1) / 2;
    tsq::DevBuf ids;
    cudaError_t e = tsq::tree_prepare(b, n, &A);
    if (e == cudaSuccess) e = ids.ensure(size_t(npairs) * 8);
    int32_t *d_ident = ids.as<int32_t>(), *d_cols = d_ident + npairs;
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_ident, n_ident, size_t(npairs) * 4, cudaMemcpyHostToDevice, b.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_cols, n_cols, size_t(npairs) * 4, cudaMemcpyHostToDevice, b.stream);
    if (e == cudaSuccess) {
      tsq::tree_error_reset_kernel<<<1, 1, 0, b.stream>>>(A.st);
      tsq::tree_init_kernel<<<dim3((n + 255) / 256, n), 256, 0, b.stream>>>(A.D, n, d_ident, d_cols, 1, nullptr,
                                                                            A.st);
      e = cudaGetLastError();
    }
    if (e != cudaSuccess) return tsq::cuda_status(e);
    rc = tsq::tree_run(A, method, b.stream, out);
    cudaStreamSynchronize(b.stream);  // `ids` is released on return
    return rc;
  } catch (const std::bad_alloc &) {
    return TSQ_E_NOMEM;
  }
}

int tsq_batch_guide_tree(tsq_batch *bt, int32_t n, int32_t method, tsq_tree_node *out) {
  if (!bt || n < 1 || n > tsq::kMaxTreeLeaves || tsq::bad_method(method) || (n > 1 && !out))
    return TSQ_E_INVALID_ARG;
  if (bt->out_mode == tsq::kOutScore || int64_t(n) * (n - 1) / 2 != bt->n || !bt->has_run) return TSQ_E_INVALID_ARG;
  if (n == 1) return TSQ_OK;
  // The batch must be the all-vs-all of n sequences in row-major pair order:
  // every pair (i, j) reads sequence i as a and sequence j as b.
  {
    std::vector<int64_t> off(static_cast<size_t>(n));
    std::vector<int32_t> len(static_cast<size_t>(n));
    for (int32_t s = 0; s + 1 < n; ++s) {
      const int64_t k = int64_t(s) * (2 * int64_t(n) - s - 1) / 2;  // pair (s, s + 1)
      off[size_t(s)] = bt->pairs_h[size_t(k)].a_off;
      len[size_t(s)] = bt->pairs_h[size_t(k)].a_len;
    }
    off[size_t(n - 1)] = bt->pairs_h[size_t(n - 2)].b_off;  // pair (0, n - 1)
    len[size_t(n - 1)] = bt->pairs_h[size_t(n - 2)].b_len;
    int64_t k = 0;
    for (int32_t i = 0; i < n; ++i)
      for (int32_t j = i + 1; j < n; ++j, ++k) {
        const tsq::PairDev &p = bt->pairs_h[size_t(k)];
        if (p.a_off != off[size_t(i)] || p.a_len != len[size_t(i)] || p.b_off != off[size_t(j)] ||
            p.b_len != len[size_t(j)])
          return TSQ_E_INVALID_ARG;
      }
  }
  try {
    if (cudaSetDevice(bt->device) != cudaSuccess) return TSQ_E_CUDA;
    int rc = TSQ_OK;
    tsq::TreeBufs &b = tsq::tree_cache(&rc);
    if (rc) return rc;
    tsq::TreeArgs A;
    cudaError_t e = tsq::tree_prepare(b, n, &A);
    const int32_t *res = bt->res.as<int32_t>();
    if (e == cudaSuccess) {
      // The distances are built on the batch's stream, after its run.
      tsq::tree_error_reset_kernel<<<1, 1, 0, bt->stream>>>(A.st);
      tsq::tree_init_kernel<<<dim3((n + 255) / 256, n), 256, 0, bt->stream>>>(
          A.D, n, res + offsetof(tsq::ResultDev, n_ident) / 4, res + offsetof(tsq::ResultDev, n_cols) / 4,
          int32_t(sizeof(tsq::ResultDev) / 4), res + offsetof(tsq::ResultDev, status) / 4, A.st);
      e = cudaGetLastError();
    }
    if (e != cudaSuccess) return tsq::cuda_status(e);
    return tsq::tree_run(A, method, bt->stream, out);
  } catch (const std::bad_alloc &) {
    return TSQ_E_NOMEM;
  }
}

}  // extern "C"
