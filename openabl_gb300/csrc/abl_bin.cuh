// Binning and neighbourhood-list work items, shared by the runtime's
// kernels (one launch per phase) and the persistent ensemble kernel (every
// phase of every timestep in one launch).  Each function does the work of
// one agent, slot, cell or (for the warp-wide merges) one warp's cell; the
// kernels in abl_runtime.cu map their threads onto items, the persistent
// kernel strides over them.
//
// Binning of an agent type (src/AnalysisVisitor.cpp:474-538 gives the
// environment and the cell size):
//   assign  cell index per agent, counted per cell (atomic rank);
//   scatter counting-sort placement: slot = cell_start[cell] + rank;
//   sort    every cell's run of slots in ascending agent id, so slots are in
//           (cell, id) order whatever order the atomics gave;
//   gather  slot-ordered copies of the position (as float) and the members
//           the near loops read.
// Neighbourhood lists (ordered near loops, CPrinter.cpp:148-173 visits
// neighbours in ascending index): per cell, the slots of every agent in the
// surrounding (2R+1)^dim cells in ascending agent id, built one axis at a
// time.  Level 0 is the cells' own runs; level a+1 merges, for every cell c,
// the level-a lists of the cells c - R .. c + R along axis a.  An element's
// place in a merged list is its index in its own source list plus, for every
// other source list, the number of smaller ids there (a binary search), so
// every element is written once per target list with no sorting pass.
#pragma once

#include "abl_device.cuh"

namespace ablbin {

// Folds m (this thread's largest |coordinate|) into *amax: a block-wide
// maximum first, then one atomic per block, skipped when it cannot raise the
// current value.  A per-warp atomic on the one address serialised up to
// 500 K atomics per binning of 16M agents at the L2.  Every thread of the
// block calls it.
__device__ __forceinline__ void fold_amax(float m, float *amax) {
  __shared__ float warp_max[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if (lane == 0) warp_max[w] = m;
  __syncthreads();
  if (w == 0) {
    m = lane < nw ? warp_max[lane] : 0.0f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0 && m > 0.0f && m > __ldcg(amax)) abl::atomic_max_nonneg(amax, m);
  }
}

__device__ __forceinline__ bool finite_bits(double x) {
  return ((__double_as_longlong(x) >> 52) & 0x7ff) != 0x7ff;
}
__device__ __forceinline__ bool finite_bits(float x) {
  return ((__float_as_int(x) >> 23) & 0xff) != 0xff;
}

// ------------------------------------------------------------ binning

// Grid of one replica of an ensemble: its cells are cell_base .. cell_base +
// nx*ny*nz - 1 of the segmented grid.  f32: the grid's rounding-error bound
// allows cell coordinates in FP32 (flo, finv: lo and 1 / cell size in
// float), as the runtime decides for single grids.
struct EnsGrid {
  int nx, ny, nz, R;
  int f32;
  float flo[3], finv;
  double lo[3];
  double inv_cell;
  long cell_base;
};

// Assign of ensemble agent i: cell in its replica's grid; returns the
// agent's largest |coordinate| (0 for i >= n).
template <typename Real, int DIM>
__device__ __forceinline__ float ens_bin_assign_item(long i, const Real *pos,
                                                     const int *replica_of, const EnsGrid *grids,
                                                     int *cell_of, int *cell_count,
                                                     int *local_rank, int *error) {
  float m = 0.0f;
  const EnsGrid &g = grids[replica_of[i]];
  const int dims[3] = {g.nx, g.ny, g.nz};
  int c[3] = {0, 0, 0};
  bool finite = true;
  const bool f32 = g.f32 != 0;
#pragma unroll
  for (int d = 0; d < DIM; d++) {
    const Real xr = pos[DIM * i + d];
    finite = finite && finite_bits(xr);
    const float xf = (float) xr;
    c[d] = f32 ? abl::cell_coord_f32(xf, g.flo[d], g.finv, dims[d])
               : abl::cell_coord((double) xr, g.lo[d], g.inv_cell, dims[d]);
    m = fmaxf(m, fabsf(xf));
  }
  if (!finite) atomicExch(error, ABL_E_NONFINITE);
  int cell = (int) (g.cell_base + ((long) c[2] * g.ny + c[1]) * g.nx + c[0]);
  cell_of[i] = cell;
  local_rank[i] = atomicAdd(&cell_count[cell], 1);
  return m;
}

__device__ __forceinline__ void bin_scatter_item(long i, const int *cell_of,
                                                 const int *local_rank, const int *cell_start,
                                                 int *order) {
  order[cell_start[cell_of[i]] + local_rank[i]] = (int) i;
}

// Sorts cell c's run of slots by agent id.  Together with the counting-sort
// scatter this gives the slot order sorted by (cell, agent id),
// deterministic.
__device__ __forceinline__ void cell_sort_item(long c, const int *cell_start, int *order) {
  int s = cell_start[c], e = cell_start[c + 1];
  constexpr int K = 16;
  if (e - s <= K) {
    // Short runs (nearly all): loaded together into registers, sorted by an
    // odd-even transposition network, stored back.
    const int len = e - s;
    int v[K];
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = k < len ? order[s + k] : 0x7fffffff;
#pragma unroll
    for (int p = 0; p < K; p++) {
#pragma unroll
      for (int k = p & 1; k + 1 < K; k += 2) {
        const int a = min(v[k], v[k + 1]), b = max(v[k], v[k + 1]);
        v[k] = a;
        v[k + 1] = b;
      }
    }
#pragma unroll
    for (int k = 0; k < K; k++)
      if (k < len) order[s + k] = v[k];
    return;
  }
  // Longer runs: insertion sort.
  for (int i = s + 1; i < e; i++) {
    int v = order[i];
    int j = i - 1;
    while (j >= s && order[j] > v) {
      order[j + 1] = order[j];
      j--;
    }
    order[j + 1] = v;
  }
}

// Slot-ordered copies: float positions and the requested member columns.
struct GatherArgs {
  int nmem;
  const void *src[ABL_MAX_MEMBERS];
  void *dst[ABL_MAX_MEMBERS];
  int bytes[ABL_MAX_MEMBERS];
  // Up to four members of 16 bytes each (float2 of doubles, e.g. boids2d's
  // pos and velocity): all loads issued before the stores.  pos16 is the
  // position's place among them (-1: not gathered, or 3D).
  int all16;
  int pos16;
};

template <typename Real, int DIM>
__device__ __forceinline__ void gather_item(long s, const int *order, const Real *pos,
                                            float *posf, const GatherArgs &g) {
  long i = order[s];
  if (g.all16) {
    uint4 v[4];
#pragma unroll
    for (int k = 0; k < 4; k++)
      if (k < g.nmem) v[k] = ABL_LDG((const uint4 *) g.src[k] + i);
    if (posf && g.pos16 >= 0 && DIM == 2) {
      uint4 p = v[0];
#pragma unroll
      for (int k = 1; k < 4; k++)
        if (k == g.pos16) p = v[k];
      posf[2 * s] = (float) __hiloint2double((int) p.y, (int) p.x);
      posf[2 * s + 1] = (float) __hiloint2double((int) p.w, (int) p.z);
    } else if (posf) {
#pragma unroll
      for (int d = 0; d < DIM; d++) posf[DIM * s + d] = (float) pos[DIM * i + d];
    }
#pragma unroll
    for (int k = 0; k < 4; k++)
      if (k < g.nmem) ((uint4 *) g.dst[k])[s] = v[k];
    return;
  }
  if (posf) {
#pragma unroll
    for (int d = 0; d < DIM; d++) posf[DIM * s + d] = (float) pos[DIM * i + d];
  }
  for (int k = 0; k < g.nmem; k++) {
    int b = g.bytes[k];
    if ((b & 7) == 0) {
      const uint64_t *src = (const uint64_t *) g.src[k] + (b / 8) * i;
      uint64_t *dst = (uint64_t *) g.dst[k] + (b / 8) * s;
      for (int w = 0; w < b / 8; w++) dst[w] = src[w];
    } else if ((b & 3) == 0) {
      const uint32_t *src = (const uint32_t *) g.src[k] + (b / 4) * i;
      uint32_t *dst = (uint32_t *) g.dst[k] + (b / 4) * s;
      for (int w = 0; w < b / 4; w++) dst[w] = src[w];
    } else {
      const uint8_t *src = (const uint8_t *) g.src[k] + b * i;
      uint8_t *dst = (uint8_t *) g.dst[k] + b * s;
      for (int w = 0; w < b; w++) dst[w] = src[w];
    }
  }
}

// ------------------------------------------------- neighbourhood lists

// Cell geometry of a single grid.
struct GridGeom {
  int nx, ny, nz, R;
  __device__ void locate(long, long &base, int &gx, int &gy, int &gz, int &r) const {
    base = 0;
    gx = nx;
    gy = ny;
    gz = nz;
    r = R;
  }
};

// Cell geometry of a segmented grid: each replica's cells in its own block.
struct EnsGeom {
  const int *cell_replica;
  const EnsGrid *grids;
  __device__ void locate(long c, long &base, int &gx, int &gy, int &gz, int &r) const {
    const EnsGrid &g = grids[cell_replica[c]];
    base = g.cell_base;
    gx = g.nx;
    gy = g.ny;
    gz = g.nz;
    r = g.R;
  }
};

// Coordinates of a cell within its grid (32-bit: grids have < 2^30 cells).
struct CellPos {
  int x[3], n[3];
  int stride[3];
  int R;
};

template <typename G>
__device__ inline CellPos cell_pos(const G &geo, long c) {
  long base;
  int nx, ny, nz, R;
  geo.locate(c, base, nx, ny, nz, R);
  CellPos p;
  const int l = (int) (c - base);
  const int nxy = nx * ny;
  p.x[2] = l / nxy;
  const int r = l - p.x[2] * nxy;
  p.x[1] = r / nx;
  p.x[0] = r - p.x[1] * nx;
  p.n[0] = nx;
  p.n[1] = ny;
  p.n[2] = nz;
  p.stride[0] = 1;
  p.stride[1] = nx;
  p.stride[2] = nxy;
  p.R = R;
  return p;
}

// Neighbour of cell c (at p) at offset d along AXIS, or -1 outside the grid.
template <int AXIS>
__device__ inline long axis_neighbour(const CellPos &p, long c, int d) {
  const int k = p.x[AXIS] + d;
  if (k < 0 || k >= p.n[AXIS]) return -1;
  return c + (long) d * p.stride[AXIS];
}

// Per cell: number of candidates in the 2R+1 source lists along AXIS.
template <typename G, int AXIS>
__device__ __forceinline__ void sep_count_item(long c, const G &geo, const int *src_off,
                                               int *dst_cnt) {
  const CellPos p = cell_pos(geo, c);
  int cnt = 0;
  for (int d = -p.R; d <= p.R; d++) {
    const long u = axis_neighbour<AXIS>(p, c, d);
    if (u >= 0) cnt += src_off[u + 1] - src_off[u];
  }
  dst_cnt[c] = cnt;
}

// Source lists of one level.  Level 0: the binned slots themselves (list of
// cell u = slots off[u] .. off[u+1]); later levels store one element per
// entry: (id, slot, float x, float y), the float position of the slot being
// what the radius prefilter reads.
struct SepSrc {
  const int *off;     // ncells + 1
  const int *order;   // level 0: slot -> id
  const float *posf;  // level 0: slot -> float position (dim per slot)
  int dim;
  const int4 *elem;   // later levels
};

constexpr int kSepMaxSrc = 7;    // source lists per target: 2R + 1 for R <= 3
constexpr int kSepWarps = 8;     // target cells (warps) per block of the warp merge kernels
constexpr int kSepThreads = 128; // target cells (threads) per block of k_sep_merge
constexpr int kSepStage = 512;   // source ids a warp of the warp merge stages

template <bool LEVEL0>
__device__ __forceinline__ int4 sep_elem_t(const SepSrc &S, int e) {
  if (!LEVEL0) return ABL_LDG(&S.elem[e]);
  return make_int4(ABL_LDG(&S.order[e]), e, __float_as_int(ABL_LDG(&S.posf[S.dim * e])),
                   __float_as_int(ABL_LDG(&S.posf[S.dim * e + 1])));
}

__device__ __forceinline__ int4 sep_elem(const SepSrc &S, int e) {
  return S.elem ? sep_elem_t<false>(S, e) : sep_elem_t<true>(S, e);
}

__device__ inline int lower_bound_src(const SepSrc &S, int b, int len, int id) {
  int lo = 0, hi = len;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (sep_elem(S, b + mid).x < id) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Source lists of target cell t along AXIS: begin and length per offset
// -R .. R (length 0 outside the grid).  Returns the total length.
template <int AXIS>
__device__ inline int sep_sources(const CellPos &P, long t, const SepSrc &S, int *b, int *n) {
  int total = 0;
#pragma unroll
  for (int k = 0; k < kSepMaxSrc; k++) {
    b[k] = 0;
    n[k] = 0;
    const int d = k - P.R;
    if (d > P.R) continue;
    const long u = axis_neighbour<AXIS>(P, t, d);
    if (u < 0) continue;
    b[k] = S.off[u];
    n[k] = S.off[u + 1] - b[k];
    total += n[k];
  }
  return total;
}

// A three-way merge of the id-sorted source lists pos[k] .. end[k], by one
// thread.  Writes elements (dst_elem) or, for the last level, slots only
// (dst_slot).
template <bool LEVEL0>
__device__ void seq_merge3(const SepSrc &S, int *pos, const int *end, int total, long out0,
                           int4 *dst_elem, int *dst_slot) {
  const int kNone = 0x7fffffff;
  int4 h[3];
#pragma unroll
  for (int k = 0; k < 3; k++)
    h[k] = pos[k] < end[k] ? sep_elem_t<LEVEL0>(S, pos[k]) : make_int4(kNone, 0, 0, 0);
  for (int q = 0; q < total; q++) {
    const bool a01 = h[0].x < h[1].x;
    const int m01 = a01 ? h[0].x : h[1].x;
    const int k = h[2].x < m01 ? 2 : (a01 ? 0 : 1);
    const int4 v = k == 0 ? h[0] : (k == 1 ? h[1] : h[2]);
    if (dst_elem) dst_elem[out0 + q] = v;
    else dst_slot[out0 + q] = v.y;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      if (j == k) {
        const int e = ++pos[j];
        h[j] = e < end[j] ? sep_elem_t<LEVEL0>(S, e) : make_int4(kNone, 0, 0, 0);
      }
    }
  }
}

// Target cell t with R = 1 merged by one thread (short lists: level 0).
template <typename G, int AXIS, bool LEVEL0>
__device__ __forceinline__ void sep_merge_item(long t, const G &geo, const SepSrc &S,
                                               const int *dst_off, int4 *dst_elem,
                                               int *dst_slot) {
  const CellPos P = cell_pos(geo, t);
  const long out0 = dst_off[t];
  const int total = (int) (dst_off[t + 1] - out0);
  if (P.R != 1 || total == 0) return;
  int pos[3], end[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const long u = axis_neighbour<AXIS>(P, t, k - 1);
    pos[k] = u >= 0 ? S.off[u] : 0;
    end[k] = u >= 0 ? S.off[u + 1] : 0;
  }
  seq_merge3<LEVEL0>(S, pos, end, total, out0, dst_elem, dst_slot);
}

// Target cell t with R = 1 merged by one warp (every lane calls it with the
// same t; `my` is the warp's kSepStage ints of shared memory).  The ids of
// the three source lists are staged with coalesced loads; an element's place
// is its index in its own list plus the number of smaller ids in the other
// two (binary searches in shared memory; the lists hold different agents),
// so the loads are independent instead of a chain of one per merged element.
// Cells whose sources exceed the staging area are merged by one lane.
// Cells of grids with R > 1 are left to sep_merge_large_item.
template <typename G, int AXIS, bool LEVEL0>
__device__ __forceinline__ void sep_merge_warp_item(long t, int lane, const G &geo,
                                                    const SepSrc &S, const int *dst_off,
                                                    int4 *dst_elem, int *dst_slot, int *my) {
  const CellPos P = cell_pos(geo, t);
  const long out0 = dst_off[t];
  const int total = (int) (dst_off[t + 1] - out0);
  if (P.R != 1 || total == 0) return;  // uniform over the warp, as is every exit below
  int b[3], n[3], st[3];
  int staged = 0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const long u = axis_neighbour<AXIS>(P, t, k - 1);
    b[k] = u >= 0 ? S.off[u] : 0;
    n[k] = u >= 0 ? S.off[u + 1] - b[k] : 0;
    st[k] = staged;
    staged += n[k];
  }
  if (staged > kSepStage) {
    if (lane == 0) {
      int pos[3] = {b[0], b[1], b[2]}, end[3] = {b[0] + n[0], b[1] + n[1], b[2] + n[2]};
      seq_merge3<LEVEL0>(S, pos, end, total, out0, dst_elem, dst_slot);
    }
    return;
  }
#pragma unroll
  for (int k = 0; k < 3; k++) {
    for (int j = lane; j < n[k]; j += 32)
      my[st[k] + j] = LEVEL0 ? ABL_LDG(&S.order[b[k] + j]) : ABL_LDG(&S.elem[b[k] + j].x);
  }
  __syncwarp();
#pragma unroll
  for (int k = 0; k < 3; k++) {
    for (int j = lane; j < n[k]; j += 32) {
      const int4 v = sep_elem_t<LEVEL0>(S, b[k] + j);
      int rank = j;
#pragma unroll
      for (int k2 = 0; k2 < 3; k2++) {
        if (k2 == k) continue;
        int lo = 0, len = n[k2];
        const int *a = my + st[k2];
        while (len > 0) {
          const int half = len >> 1;
          if (a[lo + half] < v.x) {
            lo += half + 1;
            len -= half + 1;
          } else {
            len = half;
          }
        }
        rank += lo;
      }
      if (dst_elem) dst_elem[out0 + rank] = v;
      else dst_slot[out0 + rank] = v.y;
    }
  }
}

// Target cell t of a grid with R > 1, merged by one warp: an element's place
// is its index in its own source list plus a binary search in every other
// source list.
template <typename G, int AXIS>
__device__ __forceinline__ void sep_merge_large_item(long t, int lane, const G &geo,
                                                     const SepSrc &S, const int *dst_off,
                                                     int4 *dst_elem, int *dst_slot) {
  const CellPos P = cell_pos(geo, t);
  if (P.R == 1) return;
  int b[kSepMaxSrc], n[kSepMaxSrc];
  sep_sources<AXIS>(P, t, S, b, n);
  const long out = dst_off[t];
#pragma unroll
  for (int k = 0; k < kSepMaxSrc; k++) {
    for (int j = lane; j < n[k]; j += 32) {
      const int4 v = sep_elem(S, b[k] + j);
      int rank = j;
#pragma unroll
      for (int k2 = 0; k2 < kSepMaxSrc; k2++) {
        if (k2 != k && n[k2] > 0) rank += lower_bound_src(S, b[k2], n[k2], v.x);
      }
      if (dst_elem) dst_elem[out + rank] = v;
      else dst_slot[out + rank] = v.y;
    }
  }
}

}  // namespace ablbin
