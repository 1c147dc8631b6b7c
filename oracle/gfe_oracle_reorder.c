/*
 * gfe_oracle_reorder.c -- TEST INFRASTRUCTURE ONLY (the oracle), not part of the product.
 *
 * CPU restatement of Gridap.jl v0.20.8's free-dof reordering: compute_adjacency
 * (Arrays/Tables.jl:1053-1107, with inverse_table Arrays/Tables.jl:413-445), Reverse
 * Cuthill-McKee with George-Liu pseudo-peripheral nodes (FESpaces/FESpaceReindexing.jl:31-
 * 122) and Sloan's algorithm (FESpaces/FESpaceReindexing.jl:124-262). Every loop follows the
 * Julia code step by step (queue order, tie breaks, the lazy-deletion binary heap), so the
 * permutations are the ones Gridap returns. Row sorts by degree are stable (Julia's default
 * sort), with rows first sorted by dof id as compute_adjacency leaves them.
 * All ids here are 1-based like Gridap's; iperm[old-1] = new.
 */
#include "gfe_oracle.h"

#include <limits.h>
#include <stdlib.h>
#include <string.h>

static int cmp_i32_asc(const void* a, const void* b) {
  const int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
  return (x > y) - (x < y);
}

/* Adjacency of the free dofs through the cells: row i (1-based) lists the distinct positive
 * j != i that share a cell with i, ascending. ptrs (nfree+1, 1-based like Gridap's Table)
 * and data are malloc'd; returns 0 or -1. */
int orc_compute_adjacency(int64_t ncells, int nd, const int32_t* cell_dofs, int64_t nfree,
                          int64_t** ptrs_out, int32_t** data_out) {
  /* inverse table: dof -> cells (ascending) */
  int64_t* dptr = (int64_t*)calloc((size_t)nfree + 2, sizeof(int64_t));
  if (!dptr) return -1;
  for (int64_t k = 0; k < ncells * nd; ++k)
    if (cell_dofs[k] > 0) dptr[cell_dofs[k] + 1]++;
  dptr[1] = 1;
  for (int64_t i = 1; i <= nfree; ++i) dptr[i + 1] += dptr[i];
  int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * ((size_t)nfree + 2));
  int32_t* d2c = (int32_t*)malloc(sizeof(int32_t) * ((size_t)(dptr[nfree + 1] - 1) + 1));
  if (!fill || !d2c) return -1;
  memcpy(fill, dptr, sizeof(int64_t) * ((size_t)nfree + 2));
  for (int64_t c = 0; c < ncells; ++c)
    for (int l = 0; l < nd; ++l) {
      const int32_t b = cell_dofs[c * nd + l];
      if (b > 0) d2c[fill[b]++ - 1] = (int32_t)(c + 1);
    }
  /* upper bound rows */
  int64_t* ub = (int64_t*)malloc(sizeof(int64_t) * ((size_t)nfree + 2));
  if (!ub) return -1;
  ub[1] = 1;
  for (int64_t i = 1; i <= nfree; ++i) ub[i + 1] = ub[i] + (dptr[i + 1] - dptr[i]) * nd;
  int32_t* ubd = (int32_t*)malloc(sizeof(int32_t) * ((size_t)(ub[nfree + 1] - 1) + 1));
  int64_t* fe = (int64_t*)malloc(sizeof(int64_t) * ((size_t)nfree + 2));
  if (!ubd || !fe) return -1;
  for (int64_t i = 1; i <= nfree; ++i) {
    fe[i] = ub[i];
    for (int64_t k = dptr[i]; k < dptr[i + 1]; ++k) {
      const int64_t c = d2c[k - 1] - 1;
      for (int l = 0; l < nd; ++l) {
        const int32_t j = cell_dofs[c * nd + l];
        if (j > 0 && j != i) ubd[fe[i]++ - 1] = j;
      }
    }
  }
  int64_t* ptrs = (int64_t*)malloc(sizeof(int64_t) * ((size_t)nfree + 1));
  if (!ptrs) return -1;
  ptrs[0] = 1;
  for (int64_t i = 1; i <= nfree; ++i) {
    qsort(ubd + ub[i] - 1, (size_t)(fe[i] - ub[i]), sizeof(int32_t), cmp_i32_asc);
    int64_t n = 0;
    int32_t prev = 0;
    for (int64_t k = ub[i]; k < fe[i]; ++k)
      if (ubd[k - 1] != prev) {
        ++n;
        prev = ubd[k - 1];
      }
    ptrs[i] = ptrs[i - 1] + n;
  }
  int32_t* data = (int32_t*)malloc(sizeof(int32_t) * ((size_t)(ptrs[nfree] - 1) + 1));
  if (!data) return -1;
  for (int64_t i = 1; i <= nfree; ++i) {
    int64_t p = ptrs[i - 1];
    int32_t prev = 0;
    for (int64_t k = ub[i]; k < fe[i]; ++k)
      if (ubd[k - 1] != prev) {
        data[p++ - 1] = ubd[k - 1];
        prev = ubd[k - 1];
      }
  }
  free(dptr);
  free(fill);
  free(d2c);
  free(ub);
  free(ubd);
  free(fe);
  *ptrs_out = ptrs;
  *data_out = data;
  return 0;
}

void orc_free(void* p) { free(p); }

/* ---- shared BFS with generation marks (FESpaceReindexing.jl: bfs! closures) ------------- */
typedef struct {
  int64_t n;
  const int64_t* ptrs; /* 1-based */
  const int32_t* adj;  /* 1-based ids */
  const int64_t* deg;
  int64_t* queue;      /* 1-based node ids, 1-based positions */
  int64_t* level;
  int64_t* state;      /* 0 unvisited, g visited in generation g, -1 done */
  int64_t gen;
} Bfs;

/* (qtail, last): qtail = nodes reached, last = first position of the deepest level */
static void bfs_run(Bfs* b, int64_t start, int64_t* qtail_out, int64_t* last_out) {
  const int64_t cg = ++b->gen;
  b->state[start] = cg;
  b->level[start] = 0;
  b->queue[1] = start;
  int64_t qhead = 1, qtail = 1, max_level = 0;
  while (qhead <= qtail) {
    const int64_t v = b->queue[qhead++];
    const int64_t lv = b->level[v];
    for (int64_t k = b->ptrs[v - 1]; k < b->ptrs[v]; ++k) {
      const int64_t u = b->adj[k - 1];
      /* state[u] % UInt < cg % UInt: unvisited or visited in an older generation */
      if ((uint64_t)b->state[u] < (uint64_t)cg) {
        b->state[u] = cg;
        b->level[u] = lv + 1;
        if (lv + 1 > max_level) max_level = lv + 1;
        b->queue[++qtail] = u;
      }
    }
  }
  int64_t last = qtail;
  while (last > 1 && b->level[b->queue[last - 1]] == max_level) --last;
  *qtail_out = qtail;
  *last_out = last;
}

static int64_t george_liu(Bfs* b, int64_t seed) {
  int64_t n, last;
  bfs_run(b, seed, &n, &last);
  int64_t ecc = b->level[b->queue[n]];
  int64_t current = seed;
  for (;;) {
    int64_t best = 0, best_deg = INT64_MAX;
    for (int64_t qi = last; qi <= n; ++qi) {
      const int64_t v = b->queue[qi];
      if (b->deg[v] < best_deg) {
        best_deg = b->deg[v];
        best = v;
      }
    }
    int64_t n2, last2;
    bfs_run(b, best, &n2, &last2);
    const int64_t ecc2 = b->level[b->queue[n2]];
    if (ecc2 <= ecc) return current;
    ecc = ecc2;
    n = n2;
    last = last2;
    current = best;
  }
}

/* stable sort of one row by degree (insertion sort keeps equal degrees in id order) */
static void sort_row_by_degree(int32_t* row, int64_t len, const int64_t* deg) {
  for (int64_t i = 1; i < len; ++i) {
    const int32_t v = row[i];
    int64_t j = i - 1;
    while (j >= 0 && deg[row[j]] > deg[v]) {
      row[j + 1] = row[j];
      --j;
    }
    row[j + 1] = v;
  }
}

/* Reverse Cuthill-McKee (FESpaceReindexing.jl:64-122). iperm[old-1] = new (1-based). */
int orc_rcm_perm(int64_t nfree, const int64_t* ptrs, const int32_t* adj, int64_t* iperm) {
  const size_t n1 = (size_t)nfree + 1;
  int64_t* deg = (int64_t*)calloc(n1, sizeof(int64_t));
  int32_t* sorted = (int32_t*)malloc(sizeof(int32_t) * ((size_t)(ptrs[nfree] - 1) + 1));
  int64_t* queue = (int64_t*)calloc(n1, sizeof(int64_t));
  int64_t* level = (int64_t*)calloc(n1, sizeof(int64_t));
  int64_t* state = (int64_t*)calloc(n1, sizeof(int64_t));
  int64_t* perm = (int64_t*)calloc(n1, sizeof(int64_t));
  if (!deg || !sorted || !queue || !level || !state || !perm) return -1;
  for (int64_t i = 1; i <= nfree; ++i) deg[i] = ptrs[i] - ptrs[i - 1];
  memcpy(sorted, adj, sizeof(int32_t) * (size_t)(ptrs[nfree] - 1));
  for (int64_t i = 1; i <= nfree; ++i)
    sort_row_by_degree(sorted + ptrs[i - 1] - 1, ptrs[i] - ptrs[i - 1], deg);
  Bfs b = {nfree, ptrs, sorted, deg, queue, level, state, 0};
  int64_t idx = 1;
  while (idx <= nfree) {
    int64_t seed = 0, seed_deg = INT64_MAX;
    for (int64_t i = 1; i <= nfree; ++i)
      if (state[i] == 0 && deg[i] < seed_deg) {
        seed_deg = deg[i];
        seed = i;
      }
    const int64_t peripheral = george_liu(&b, seed);
    int64_t n, last;
    bfs_run(&b, peripheral, &n, &last);
    for (int64_t qi = 1; qi <= n; ++qi) {
      const int64_t v = queue[qi];
      state[v] = -1;
      perm[idx++] = v;
    }
  }
  for (int64_t i = 1; i <= nfree; ++i) iperm[perm[nfree + 1 - i] - 1] = i; /* reverse! */
  free(deg);
  free(sorted);
  free(queue);
  free(level);
  free(state);
  free(perm);
  return 0;
}

/* ---- Sloan (FESpaceReindexing.jl:124-262) ------------------------------------------------ */
typedef struct {
  int64_t pr, node;
} HeapItem;

typedef struct {
  HeapItem* h;
  int64_t n, cap;
  int64_t* f;
} Heap;

static int heap_push(Heap* H, int64_t node, int64_t pr) {
  H->f[node] = pr;
  if (H->n == H->cap) {
    H->cap = H->cap ? 2 * H->cap : 1024;
    HeapItem* nh = (HeapItem*)realloc(H->h, sizeof(HeapItem) * (size_t)H->cap);
    if (!nh) return -1;
    H->h = nh;
  }
  HeapItem* h = H->h - 1; /* 1-based */
  h[++H->n] = (HeapItem){pr, node};
  int64_t i = H->n;
  while (i > 1) {
    const int64_t p = i >> 1;
    if (h[p].pr >= h[i].pr) break;
    const HeapItem t = h[p];
    h[p] = h[i];
    h[i] = t;
    i = p;
  }
  return 0;
}

static void heap_siftdown(Heap* H) {
  HeapItem* h = H->h - 1;
  int64_t i = 1;
  const int64_t n = H->n;
  for (;;) {
    int64_t c = 2 * i;
    if (c > n) break;
    if (c + 1 <= n && h[c + 1].pr > h[c].pr) ++c;
    if (h[c].pr <= h[i].pr) break;
    const HeapItem t = h[c];
    h[c] = h[i];
    h[i] = t;
    i = c;
  }
}

static int64_t heap_pop(Heap* H) {
  HeapItem* h = H->h - 1;
  while (H->n > 0) {
    const HeapItem top = h[1];
    if (H->n == 1) {
      H->n = 0;
    } else {
      h[1] = h[H->n--];
      heap_siftdown(H);
    }
    if (H->f[top.node] == top.pr) return top.node;
  }
  return 0;
}

int orc_sloan_perm(int64_t nfree, const int64_t* ptrs, const int32_t* adj, int64_t w1,
                   int64_t w2, int64_t* iperm) {
  const size_t n1 = (size_t)nfree + 1;
  int64_t* deg = (int64_t*)calloc(n1, sizeof(int64_t));
  int64_t* queue = (int64_t*)calloc(n1, sizeof(int64_t));
  int64_t* level = (int64_t*)calloc(n1, sizeof(int64_t));
  int64_t* state = (int64_t*)calloc(n1, sizeof(int64_t));
  int64_t* perm = (int64_t*)calloc(n1, sizeof(int64_t));
  int64_t* dist = (int64_t*)calloc(n1, sizeof(int64_t));
  int64_t* f = (int64_t*)malloc(sizeof(int64_t) * n1);
  int64_t* c = (int64_t*)calloc(n1, sizeof(int64_t));
  int8_t* status = (int8_t*)calloc(n1, 1);
  if (!deg || !queue || !level || !state || !perm || !dist || !f || !c || !status) return -1;
  for (size_t i = 0; i < n1; ++i) f[i] = INT64_MIN;
  for (int64_t i = 1; i <= nfree; ++i) deg[i] = ptrs[i] - ptrs[i - 1];
  Bfs b = {nfree, ptrs, adj, deg, queue, level, state, 0};
  Heap H = {NULL, 0, 0, f};
  int64_t idx = 1;
  while (idx <= nfree) {
    int64_t seed = 0, seed_deg = INT64_MAX;
    for (int64_t i = 1; i <= nfree; ++i)
      if (status[i] == 0 && deg[i] < seed_deg) {
        seed_deg = deg[i];
        seed = i;
      }
    const int64_t E = george_liu(&b, seed);
    int64_t n_comp, last_e;
    bfs_run(&b, E, &n_comp, &last_e);
    int64_t S = 0, S_deg = INT64_MAX, max_dist = 0, max_deg = 0;
    for (int64_t qi = 1; qi <= n_comp; ++qi) {
      const int64_t v = queue[qi];
      dist[v] = level[v];
      if (level[v] > max_dist) max_dist = level[v];
      if (deg[v] > max_deg) max_deg = deg[v];
      if (qi >= last_e && deg[v] < S_deg) {
        S_deg = deg[v];
        S = v;
      }
    }
    const int64_t ew1 = w1 * (max_deg > 1 ? max_deg : 1);
    const int64_t ew2 = w2 * (max_dist > 1 ? max_dist : 1);
    status[S] = 1;
    c[S] = 0;
    if (heap_push(&H, S, ew1 * dist[S])) return -1;
    int64_t done = 0;
    while (done < n_comp) {
      const int64_t v = heap_pop(&H);
      if (v == 0) break;
      if (status[v] == 1) {
        status[v] = 2;
        for (int64_t k = ptrs[v - 1]; k < ptrs[v]; ++k) {
          const int64_t u = adj[k - 1];
          if (status[u] == 0) {
            status[u] = 1;
            int64_t cu = 0;
            for (int64_t k2 = ptrs[u - 1]; k2 < ptrs[u]; ++k2) {
              const int64_t w = adj[k2 - 1];
              if (status[w] == 1 || status[w] == 2) {
                ++cu;
                ++c[w];
                if (heap_push(&H, w, ew1 * dist[w] + ew2 * c[w])) return -1;
              }
            }
            c[u] = cu;
            if (heap_push(&H, u, ew1 * dist[u] + ew2 * cu)) return -1;
          }
        }
        if (heap_push(&H, v, ew1 * dist[v] + ew2 * c[v])) return -1;
      } else if (status[v] == 2) {
        status[v] = 3;
        f[v] = INT64_MIN;
        perm[idx++] = v;
        ++done;
      }
    }
    for (int64_t qi = 1; qi <= n_comp; ++qi) state[queue[qi]] = -1;
  }
  for (int64_t i = 1; i <= nfree; ++i) iperm[perm[i] - 1] = i;
  free(deg);
  free(queue);
  free(level);
  free(state);
  free(perm);
  free(dist);
  free(f);
  free(c);
  free(status);
  free(H.h);
  return 0;
}
