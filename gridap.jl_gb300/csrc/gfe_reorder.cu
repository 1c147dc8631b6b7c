// gfe_reorder.cu -- free-dof permutations of Gridap's reindex_free_dof_ids
// (FESpaces/FESpaceReindexing.jl:264-343): Reverse Cuthill-McKee with George-Liu
// pseudo-peripheral nodes, and Sloan's wavefront ordering.
//
// The dof adjacency is the sparsity pattern of the cell dofs without its diagonal, built on
// the device by the symbolic loop (the same lists Gridap's compute_adjacency returns,
// Arrays/Tables.jl:1053-1107). Every breadth-first search runs level-synchronously on the
// device and still yields the sequential queue order: a node of level L+1 enters the queue
// when its first-queued level-L neighbour is processed, and the children of one parent come
// in the order of the parent's adjacency row -- ascending (degree, id) for Cuthill-McKee,
// whose rows are stably sorted by degree, ascending id for Sloan. So level L+1 is the
// level's nodes sorted by (queue position of the first parent, degree or 0, id):
//   expand   one thread per level-L node claims unvisited neighbours (atomicCAS on the
//            level) and lowers their parent position (atomicMin);
//   bucket   counting sort by parent position (count, scan, fill), then each parent's
//            bucket -- at most its degree -- sorted by (degree, id) or id by one thread.
// The host reads one count per level. Sloan's numbering loop (a lazy-deletion binary heap
// over a moving front) is inherently sequential and runs on the host over the device-built
// adjacency, with the BFS distances from the device.
#include <algorithm>
#include <climits>
#include <vector>

#include "gfe_internal.h"

namespace gfe {
namespace {

constexpr int kB = 256;

// level -1 = unvisited in this search, -2 = numbered in an earlier component
__global__ void k_bfs_init(int64_t n, const uint8_t* __restrict__ done, int32_t* __restrict__ lev,
                           int32_t* __restrict__ par) {
  for (int64_t i = (int64_t)blockIdx.x * kB + threadIdx.x; i < n; i += (int64_t)gridDim.x * kB) {
    lev[i] = done[i] ? -2 : -1;
    par[i] = INT_MAX;
  }
}

__global__ void k_bfs_root(int32_t r, int32_t* lev, int32_t* pos, int32_t* queue) {
  lev[r] = 0;
  pos[r] = 0;
  queue[0] = r;
}

// frontier = queue[head, head+m): claim unvisited neighbours for level L+1
__global__ void k_bfs_expand(const int32_t* __restrict__ queue, int32_t head, int32_t m,
                             int32_t L, const int32_t* __restrict__ rowptr,
                             const int32_t* __restrict__ colval, int32_t* __restrict__ lev,
                             int32_t* __restrict__ par, int32_t* __restrict__ next,
                             int32_t* __restrict__ cnt) {
  const int32_t t = blockIdx.x * kB + threadIdx.x;
  if (t >= m) return;
  const int32_t p = head + t;
  const int32_t v = queue[p];
  for (int32_t k = rowptr[v]; k < rowptr[v + 1]; ++k) {
    const int32_t u = colval[k];
    if (u == v) continue;
    const int32_t lu = lev[u];
    if (lu != -1 && lu != L + 1) continue;
    const int32_t old = atomicCAS(&lev[u], -1, L + 1);
    if (old == -1) next[atomicAdd(cnt, 1)] = u;
    if (old == -1 || old == L + 1) atomicMin(&par[u], p);
  }
}

__global__ void k_bucket_count(const int32_t* __restrict__ next, int32_t m,
                               const int32_t* __restrict__ par, int32_t head,
                               int32_t* __restrict__ bcnt) {
  const int32_t t = blockIdx.x * kB + threadIdx.x;
  if (t < m) atomicAdd(&bcnt[par[next[t]] - head], 1);
}

__global__ void k_bucket_fill(const int32_t* __restrict__ next, int32_t m,
                              const int32_t* __restrict__ par, int32_t head,
                              const int64_t* __restrict__ boff, int32_t* __restrict__ bfill,
                              int32_t* __restrict__ out) {
  const int32_t t = blockIdx.x * kB + threadIdx.x;
  if (t >= m) return;
  const int32_t u = next[t];
  const int32_t b = par[u] - head;
  out[boff[b] + atomicAdd(&bfill[b], 1)] = u;
}

// one thread per parent: its children sorted by (degree, id) (by_degree) or by id
__global__ void k_bucket_sort(int32_t nb, const int64_t* __restrict__ boff,
                              int32_t* __restrict__ out, const int32_t* __restrict__ rowptr,
                              bool by_degree) {
  const int32_t b = blockIdx.x * kB + threadIdx.x;
  if (b >= nb) return;
  const int64_t s = boff[b], e = boff[b + 1];
  for (int64_t i = s + 1; i < e; ++i) {
    const int32_t u = out[i];
    const int32_t du = by_degree ? rowptr[u + 1] - rowptr[u] : 0;
    int64_t j = i - 1;
    while (j >= s) {
      const int32_t w = out[j];
      const int32_t dw = by_degree ? rowptr[w + 1] - rowptr[w] : 0;
      if (dw < du || (dw == du && w < u)) break;
      out[j + 1] = w;
      --j;
    }
    out[j + 1] = u;
  }
}

__global__ void k_set_pos(const int32_t* __restrict__ queue, int32_t start, int32_t m,
                          int32_t* __restrict__ pos) {
  const int32_t t = blockIdx.x * kB + threadIdx.x;
  if (t < m) pos[queue[start + t]] = start + t;
}

// argmin of (degree, id) over the nodes not yet numbered
__global__ void k_seed(int64_t n, const uint8_t* __restrict__ done,
                       const int32_t* __restrict__ rowptr, unsigned long long* best) {
  for (int64_t i = (int64_t)blockIdx.x * kB + threadIdx.x; i < n; i += (int64_t)gridDim.x * kB)
    if (!done[i]) {
      const unsigned long long key =
          ((unsigned long long)(rowptr[i + 1] - rowptr[i]) << 32) | (unsigned long long)i;
      atomicMin(best, key);
    }
}

// argmin of (degree, queue position) over queue[s, e)
__global__ void k_min_degree_in(const int32_t* __restrict__ queue, int32_t s, int32_t e,
                                const int32_t* __restrict__ rowptr, unsigned long long* best) {
  const int32_t p = s + blockIdx.x * kB + threadIdx.x;
  if (p >= e) return;
  const int32_t v = queue[p];
  const unsigned long long key =
      ((unsigned long long)(rowptr[v + 1] - rowptr[v]) << 32) | (unsigned long long)p;
  atomicMin(best, key);
}

__global__ void k_number(const int32_t* __restrict__ queue, int32_t n, int64_t idx,
                         int32_t* __restrict__ perm, uint8_t* __restrict__ done) {
  const int32_t t = blockIdx.x * kB + threadIdx.x;
  if (t >= n) return;
  perm[idx + t] = queue[t];
  done[queue[t]] = 1;
}

}  // namespace

namespace {

struct DeviceBfs {
  gfe_ctx* ctx;
  int64_t n;
  const int32_t* rowptr;
  const int32_t* colval;
  bool by_degree;
  DevBuf buf;
  int32_t *lev, *par, *pos, *queue, *next, *bcnt, *bfill, *perm, *cnt;
  int64_t* boff;
  uint8_t* done;
  unsigned long long* best;
  std::vector<int32_t> level_start;  // queue position where each level starts (+ end)

  explicit DeviceBfs(gfe_ctx* c) : ctx(c), buf(c) {}

  int init(int64_t nn, const int32_t* rp, const int32_t* cv) {
    n = nn;
    rowptr = rp;
    colval = cv;
    const size_t n1 = (size_t)(n > 0 ? n : 1) + 1;
    GFE_TRY(buf.reserve(n1 * (4 * 9 + 8 + 1) + 256));
    char* p = (char*)buf.ptr;
    auto take = [&](size_t bytes) {
      char* r = p;
      p += (bytes + 15) & ~(size_t)15;
      return r;
    };
    lev = (int32_t*)take(4 * n1);
    par = (int32_t*)take(4 * n1);
    pos = (int32_t*)take(4 * n1);
    queue = (int32_t*)take(4 * n1);
    next = (int32_t*)take(4 * n1);
    bcnt = (int32_t*)take(4 * n1);
    bfill = (int32_t*)take(4 * n1);
    perm = (int32_t*)take(4 * n1);
    cnt = (int32_t*)take(16);
    boff = (int64_t*)take(8 * n1);
    best = (unsigned long long*)take(16);
    done = (uint8_t*)take(n1);
    GFE_CUDA_TRY(cudaMemsetAsync(done, 0, n1, ctx->stream));
    return GFE_OK;
  }

  unsigned grid(int64_t m) const { return (unsigned)std::max<int64_t>(1, (m + kB - 1) / kB); }

  // BFS from root over the nodes not numbered yet; the queue holds the visit order.
  // Returns the number of nodes reached; level_start delimits the levels.
  int run(int32_t root, int32_t* reached) {
    k_bfs_init<<<(unsigned)std::min<int64_t>((n + kB - 1) / kB, (int64_t)ctx->num_sms * 8) + 0u,
                 kB, 0, ctx->stream>>>(n, done, lev, par);
    k_bfs_root<<<1, 1, 0, ctx->stream>>>(root, lev, pos, queue);
    ctx->launches += 2;
    level_start.assign(1, 0);
    int32_t head = 0, tail = 1, L = 0;
    while (tail > head) {
      level_start.push_back(tail);
      const int32_t m = tail - head;
      GFE_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int32_t), ctx->stream));
      k_bfs_expand<<<grid(m), kB, 0, ctx->stream>>>(queue, head, m, L, rowptr, colval, lev, par,
                                                    next, cnt);
      ctx->launches++;
      int32_t mn = 0;
      GFE_TRY(copy_out(ctx, &mn, cnt, sizeof(int32_t)));
      if (mn == 0) break;
      if ((int64_t)tail + mn > n)
        return set_error(GFE_ERR_INVALID_ARGUMENT, "dof permutation: inconsistent adjacency");
      GFE_CUDA_TRY(cudaMemsetAsync(bcnt, 0, sizeof(int32_t) * m, ctx->stream));
      GFE_CUDA_TRY(cudaMemsetAsync(bfill, 0, sizeof(int32_t) * m, ctx->stream));
      k_bucket_count<<<grid(mn), kB, 0, ctx->stream>>>(next, mn, par, head, bcnt);
      ctx->launches++;
      GFE_TRY(scan_exclusive_i32_to_i64(ctx, bcnt, boff, m));
      k_bucket_fill<<<grid(mn), kB, 0, ctx->stream>>>(next, mn, par, head, boff, bfill,
                                                      queue + tail);
      k_bucket_sort<<<grid(m), kB, 0, ctx->stream>>>(m, boff, queue + tail, rowptr, by_degree);
      k_set_pos<<<grid(mn), kB, 0, ctx->stream>>>(queue, tail, mn, pos);
      ctx->launches += 3;
      GFE_CUDA_TRY(cudaGetLastError());
      head = tail;
      tail += mn;
      ++L;
    }
    *reached = tail;
    return GFE_OK;
  }

  // (degree, position)-first node of queue[s, e)
  int min_degree_in(int32_t s, int32_t e, int32_t* node) {
    const unsigned long long init = ~0ull;
    GFE_CUDA_TRY(cudaMemcpyAsync(best, &init, sizeof(init), cudaMemcpyHostToDevice, ctx->stream));
    k_min_degree_in<<<grid(e - s), kB, 0, ctx->stream>>>(queue, s, e, rowptr, best);
    ctx->launches++;
    unsigned long long h = 0;
    GFE_TRY(copy_out(ctx, &h, best, sizeof(h)));
    const int32_t p = (int32_t)(h & 0xffffffffu);
    GFE_TRY(copy_out(ctx, node, queue + p, sizeof(int32_t)));
    return GFE_OK;
  }

  int seed(int32_t* node) {
    const unsigned long long init = ~0ull;
    GFE_CUDA_TRY(cudaMemcpyAsync(best, &init, sizeof(init), cudaMemcpyHostToDevice, ctx->stream));
    k_seed<<<(unsigned)std::min<int64_t>((n + kB - 1) / kB, (int64_t)ctx->num_sms * 8), kB, 0,
             ctx->stream>>>(n, done, rowptr, best);
    ctx->launches++;
    unsigned long long h = 0;
    GFE_TRY(copy_out(ctx, &h, best, sizeof(h)));
    *node = (int32_t)(h & 0xffffffffu);
    return GFE_OK;
  }

  // George-Liu pseudo-peripheral node from seed (FESpaceReindexing.jl:31-49)
  int peripheral(int32_t s, int32_t* out) {
    int32_t nreach = 0;
    GFE_TRY(run(s, &nreach));
    int32_t ecc = (int32_t)level_start.size() - 2;
    int32_t last = level_start[level_start.size() - 2];
    int32_t current = s;
    for (int it = 0; it < 1000; ++it) {
      int32_t b = 0;
      GFE_TRY(min_degree_in(last, nreach, &b));
      GFE_TRY(run(b, &nreach));
      const int32_t ecc2 = (int32_t)level_start.size() - 2;
      if (ecc2 <= ecc) break;
      ecc = ecc2;
      last = level_start[level_start.size() - 2];
      current = b;
    }
    *out = current;
    return GFE_OK;
  }
};

__global__ void k_mark_done(const int32_t* __restrict__ queue, int32_t n,
                            uint8_t* __restrict__ done) {
  const int32_t t = blockIdx.x * kB + threadIdx.x;
  if (t < n) done[queue[t]] = 1;
}

// Reverse Cuthill-McKee (FESpaceReindexing.jl:64-122) on the device.
int rcm_device(DeviceBfs& B, int64_t* iperm) {
  const int64_t n = B.n;
  B.by_degree = true;
  int64_t idx = 0;
  while (idx < n) {
    int32_t seed = 0, per = 0, reached = 0;
    GFE_TRY(B.seed(&seed));
    GFE_TRY(B.peripheral(seed, &per));
    GFE_TRY(B.run(per, &reached));
    k_number<<<B.grid(reached), kB, 0, B.ctx->stream>>>(B.queue, reached, idx, B.perm, B.done);
    B.ctx->launches++;
    GFE_CUDA_TRY(cudaGetLastError());
    idx += reached;
  }
  std::vector<int32_t> perm((size_t)n);
  GFE_TRY(copy_out(B.ctx, perm.data(), B.perm, sizeof(int32_t) * (size_t)n));
  for (int64_t i = 0; i < n; ++i) iperm[perm[(size_t)(n - 1 - i)]] = i + 1;  // reverse!
  return GFE_OK;
}

// Sloan (FESpaceReindexing.jl:124-262): peripheral node and distances from the device BFS,
// the numbering loop over a lazy-deletion max-heap on the host.
int sloan_device(DeviceBfs& B, const std::vector<int32_t>& rp, const std::vector<int32_t>& cv,
                 int64_t w1, int64_t w2, int64_t* iperm) {
  const int64_t n = B.n;
  B.by_degree = false;
  auto deg = [&](int64_t v) { return (int64_t)(rp[v + 1] - rp[v] - 1); };
  std::vector<int64_t> dist(n, 0), c(n, 0), f(n, INT64_MIN);
  std::vector<int8_t> status(n, 0);
  std::vector<std::pair<int64_t, int64_t>> heap;  // (priority, node), 0-based array
  auto push = [&](int64_t node, int64_t pr) {
    f[node] = pr;
    heap.emplace_back(pr, node);
    size_t i = heap.size();  // 1-based sift-up
    while (i > 1) {
      const size_t p = i >> 1;
      if (heap[p - 1].first >= heap[i - 1].first) break;
      std::swap(heap[p - 1], heap[i - 1]);
      i = p;
    }
  };
  auto pop = [&]() -> int64_t {
    while (!heap.empty()) {
      const auto top = heap[0];
      if (heap.size() == 1) {
        heap.pop_back();
      } else {
        heap[0] = heap.back();
        heap.pop_back();
        size_t i = 1;
        const size_t m = heap.size();
        for (;;) {
          size_t ci = 2 * i;
          if (ci > m) break;
          if (ci + 1 <= m && heap[ci].first > heap[ci - 1].first) ++ci;
          if (heap[ci - 1].first <= heap[i - 1].first) break;
          std::swap(heap[ci - 1], heap[i - 1]);
          i = ci;
        }
      }
      if (f[top.second] == top.first) return top.second;
    }
    return -1;
  };
  std::vector<int32_t> queue, lev;
  int64_t idx = 0;
  while (idx < n) {
    int32_t seed = 0, E = 0, ncomp = 0;
    GFE_TRY(B.seed(&seed));
    GFE_TRY(B.peripheral(seed, &E));
    GFE_TRY(B.run(E, &ncomp));
    const int32_t last_e = B.level_start[B.level_start.size() - 2];
    queue.resize((size_t)ncomp);
    GFE_TRY(copy_out(B.ctx, queue.data(), B.queue, sizeof(int32_t) * (size_t)ncomp));
    lev.resize((size_t)n);
    GFE_TRY(copy_out(B.ctx, lev.data(), B.lev, sizeof(int32_t) * (size_t)n));
    int64_t S = -1, S_deg = INT64_MAX, max_dist = 0, max_deg = 0;
    for (int32_t qi = 0; qi < ncomp; ++qi) {
      const int64_t v = queue[(size_t)qi];
      dist[v] = lev[(size_t)v];
      max_dist = std::max<int64_t>(max_dist, dist[v]);
      max_deg = std::max<int64_t>(max_deg, deg(v));
      if (qi >= last_e && deg(v) < S_deg) {
        S_deg = deg(v);
        S = v;
      }
    }
    const int64_t ew1 = w1 * std::max<int64_t>(max_deg, 1);
    const int64_t ew2 = w2 * std::max<int64_t>(max_dist, 1);
    status[S] = 1;
    c[S] = 0;
    push(S, ew1 * dist[S]);
    int64_t comp_done = 0;
    while (comp_done < ncomp) {
      const int64_t v = pop();
      if (v < 0) break;
      if (status[v] == 1) {
        status[v] = 2;
        for (int32_t k = rp[v]; k < rp[v + 1]; ++k) {
          const int64_t u = cv[k];
          if (u == v || status[u] != 0) continue;
          status[u] = 1;
          int64_t cu = 0;
          for (int32_t k2 = rp[u]; k2 < rp[u + 1]; ++k2) {
            const int64_t w = cv[k2];
            if (w == u) continue;
            if (status[w] == 1 || status[w] == 2) {
              ++cu;
              ++c[w];
              push(w, ew1 * dist[w] + ew2 * c[w]);
            }
          }
          c[u] = cu;
          push(u, ew1 * dist[u] + ew2 * cu);
        }
        push(v, ew1 * dist[v] + ew2 * c[v]);
      } else if (status[v] == 2) {
        status[v] = 3;
        f[v] = INT64_MIN;
        iperm[v] = ++idx;
        ++comp_done;
      }
    }
    if (comp_done != ncomp)
      return set_error(GFE_ERR_INVALID_ARGUMENT, "sloan: component numbering incomplete");
    k_mark_done<<<B.grid(ncomp), kB, 0, B.ctx->stream>>>(B.queue, ncomp, B.done);
    B.ctx->launches++;
    GFE_CUDA_TRY(cudaGetLastError());
  }
  return GFE_OK;
}

}  // namespace
}  // namespace gfe

using namespace gfe;

extern "C" int gfe_dof_permutation(gfe_ctx* ctx, int64_t ncells, int32_t nd,
                                   const int32_t* cell_dof_ids, int64_t nfree, int32_t algorithm,
                                   int32_t w1, int32_t w2, int64_t* iperm) {
  NvtxRange nvtx_range("gfe_dof_permutation");
  clear_error();
  if (!ctx || !iperm || nd < 1 || ncells < 0 || nfree < 0 || (ncells > 0 && !cell_dof_ids))
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_dof_permutation: bad arguments");
  if (algorithm != GFE_REORDER_RCM && algorithm != GFE_REORDER_SLOAN)
    return set_error(GFE_ERR_INVALID_ARGUMENT, "gfe_dof_permutation: algorithm %d", algorithm);
  if (nfree > INT32_MAX - 1)
    return set_error(GFE_ERR_UNSUPPORTED, "gfe_dof_permutation: more than 2^31 dofs");
  if (nfree == 0) return GFE_OK;
  DeviceGuard g(ctx->device);
  // adjacency = the symbolic loop's pattern (sorted rows, diagonal included)
  gfe_matrix T;
  T.ctx = ctx;
  for (DevBuf* b : {&T.rowptr, &T.colval, &T.val, &T.cell_rows, &T.cell_cols, &T.ref_ptr,
                    &T.refs, &T.refpos})
    b->owner = ctx;
  T.nrows = T.ncols = nfree;
  T.nd = nd;
  T.ncells = ncells;
  const size_t idsz = sizeof(int32_t) * (size_t)ncells * nd;
  GFE_TRY(T.cell_rows.reserve(idsz > 0 ? idsz : 4));
  GFE_TRY(T.cell_cols.reserve(idsz > 0 ? idsz : 4));
  if (idsz) {
    GFE_CUDA_TRY(cudaMemcpyAsync(T.cell_rows.ptr, cell_dof_ids, idsz, cudaMemcpyDefault,
                                 ctx->stream));
    GFE_CUDA_TRY(cudaMemcpyAsync(T.cell_cols.ptr, cell_dof_ids, idsz, cudaMemcpyDefault,
                                 ctx->stream));
  }
  GFE_TRY(build_pattern(ctx, &T));
  DeviceBfs B(ctx);
  GFE_TRY(B.init(nfree, T.rowptr.as<int32_t>(), T.colval.as<int32_t>()));
  if (algorithm == GFE_REORDER_RCM) {
    GFE_TRY(rcm_device(B, iperm));
  } else {
    std::vector<int32_t> rp((size_t)nfree + 1), cv((size_t)T.nnz);
    GFE_TRY(copy_out(ctx, rp.data(), T.rowptr.ptr, sizeof(int32_t) * rp.size()));
    GFE_TRY(copy_out(ctx, cv.data(), T.colval.ptr, sizeof(int32_t) * cv.size()));
    GFE_TRY(sloan_device(B, rp, cv, w1, w2, iperm));
  }
  return check_device_error(ctx, "gfe_dof_permutation");
}
