// OpenABL CUDA runtime: agent state, uniform-grid binning and the step loop.
//
// Per agent type the context keeps structure-of-arrays columns in two
// buffers (the reference's agents_X / agents_X_dbuf pair,
// src/backend/CPrinter.cpp:278-293).  A timestep runs the model's step
// functions in simulate order (CPrinter.cpp:196-229); each one reads the
// current buffer, writes the other, and the two are swapped afterwards.
//
// Before a step function whose body contains a `near` loop, the neighbour
// type is binned (unless its positions have not changed since the last
// binning):
//   1. assign   cell index per agent, atomically counted per cell; the
//               largest |coordinate| is reduced for the radius prefilter;
//   2. scan     exclusive prefix sum of the cell counts -> cell_start;
//   3. scatter  counting-sort placement: slot = cell_start[cell] + rank;
//   4. gather   slot-ordered copies of the position (as float, for the
//               prefilter) and of the members the near loops read;
//   5. lists    (ordered bodies only) per cell, the slots of all agents in
//               the surrounding cells sorted by agent id, so that the loop
//               body sees neighbours in the reference's ascending index order.
// Every buffer is sized from the agent count and the grid at upload time, so
// a timestep needs no host synchronisation and is captured once into a CUDA
// graph that abl_run replays.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "abl_bin.cuh"
#include "abl_device.cuh"
#include "abl_model.h"
#include "abl_persist.cuh"
#include "openabl_cuda_diag.h"

namespace {

using namespace ablbin;

constexpr int kScanBlock = 1024;

#define ABL_CUDA_TRY(expr)                                                   \
  do {                                                                       \
    cudaError_t e_ = (expr);                                                 \
    if (e_ != cudaSuccess) {                                                 \
      std::fprintf(stderr, "openabl-cuda: %s failed: %s (%s:%d)\n", #expr,   \
                   cudaGetErrorString(e_), __FILE__, __LINE__);              \
      return ABL_E_CUDA;                                                     \
    }                                                                        \
  } while (0)

#define ABL_TRY(expr)          \
  do {                         \
    int r_ = (expr);           \
    if (r_ != ABL_OK) return r_; \
  } while (0)

// ------------------------------------------------------------------ scan

// Inclusive scan of one block of kScanBlock ints (4 per thread, warp
// shuffles), writing the block total to block_sums.
__global__ void k_scan_blocks(const int *in, int *out, long m, int *block_sums) {
  __shared__ int warp_tot[kScanBlock / 4 / 32];
  long base = (long) blockIdx.x * kScanBlock;
  int t = threadIdx.x;
  int v[4];
  int run = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    long i = base + 4 * t + k;
    v[k] = i < m ? in[i] : 0;
    run += v[k];
  }
  int lane = t & 31, w = t >> 5;
  int incl = run;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_tot[w] = incl;
  __syncthreads();
  if (w == 0) {
    int nw = blockDim.x / 32;
    int x = lane < nw ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane < nw) warp_tot[lane] = x;
  }
  __syncthreads();
  int prefix = (w > 0 ? warp_tot[w - 1] : 0) + incl - run;  // exclusive for this thread
#pragma unroll
  for (int k = 0; k < 4; k++) {
    long i = base + 4 * t + k;
    prefix += v[k];
    if (i < m) out[i] = prefix;  // inclusive
  }
  if (t == blockDim.x - 1) block_sums[blockIdx.x] = warp_tot[blockDim.x / 32 - 1];
}

// Exclusive scan with total of at most kScanBlock ints in one block: out[0]
// = 0, out[i + 1] = in[0] + ... + in[i].  Replaces the block pass, the
// memset and the finishing pass of a one-block scan level.
__global__ void k_scan_single(const int *in, int *out, long m) {
  __shared__ int warp_tot[kScanBlock / 4 / 32];
  int t = threadIdx.x;
  int v[4];
  int run = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    long i = 4 * t + k;
    v[k] = i < m ? in[i] : 0;
    run += v[k];
  }
  int lane = t & 31, w = t >> 5;
  int incl = run;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_tot[w] = incl;
  __syncthreads();
  if (w == 0) {
    int nw = blockDim.x / 32;
    int x = lane < nw ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane < nw) warp_tot[lane] = x;
  }
  __syncthreads();
  int prefix = (w > 0 ? warp_tot[w - 1] : 0) + incl - run;
  if (t == 0) out[0] = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    long i = 4 * t + k;
    prefix += v[k];
    if (i < m) out[i + 1] = prefix;
  }
}

// Turns per-block inclusive scans into a global exclusive scan with total.
__global__ void k_scan_finish(const int *incl, int *out_excl, long m, const int *block_offsets) {
  long i = (long) blockIdx.x * blockDim.x + threadIdx.x;
  if (i > m) return;
  if (i == 0) {
    out_excl[0] = 0;
    return;
  }
  long j = i - 1;
  out_excl[i] = incl[j] + block_offsets[j / kScanBlock];
}

// Last pass of a scan whose block totals fit one block: thread j of a CTA
// of 256 (all in one scan block, as kScanBlock is a multiple of 256) writes
// out_excl[j + 1] = incl[j] + the totals of the scan blocks before its own,
// which the CTA adds up itself instead of a separate kernel scanning them.
__global__ void k_scan_finish_sums(const int *incl, int *out_excl, long m, const int *sums) {
  __shared__ int part[8];
  const long j0 = (long) blockIdx.x * blockDim.x;
  const int sb = (int) (j0 / kScanBlock);
  int acc = 0;
  for (int k = threadIdx.x; k < sb; k += blockDim.x) acc += sums[k];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  int off = 0;
#pragma unroll
  for (int w = 0; w < 8; w++) off += part[w];
  const long j = j0 + threadIdx.x;
  if (j == 0) out_excl[0] = 0;
  if (j < m) out_excl[j + 1] = incl[j] + off;
}

// Scan plan for an exclusive scan of m ints.  Level l scans its input in
// blocks (incl), collects the block totals (sums) and obtains the block
// offsets (offs, nb + 1 entries) by scanning the totals one level up.
struct ScanLevel {
  long m = 0, nb = 0;
  int *incl = nullptr, *sums = nullptr, *offs = nullptr;
};
struct ScanPlan {
  std::vector<ScanLevel> levels;
};

// ------------------------------------------------------------ binning


// F32: cell coordinates from the float-rounded position in FP32 (this GPU's
// FP64 pipe is narrow; the conversions to float are needed for amax anyway).
template <typename Real, int DIM, bool F32>
__global__ void k_bin_assign(const Real *pos, long n, int nx, int ny, int nz, double lo0,
                             double lo1, double lo2, double inv_cell, int *cell_of,
                             int *cell_count, int *local_rank, float *amax, int *error) {
  long i = (long) blockIdx.x * blockDim.x + threadIdx.x;
  float m = 0.0f;
  if (i < n) {
    const double lo[3] = {lo0, lo1, lo2};
    const int dims[3] = {nx, ny, nz};
    int c[3] = {0, 0, 0};
    bool finite = true;
#pragma unroll
    for (int d = 0; d < DIM; d++) {
      const Real xr = pos[DIM * i + d];
      finite = finite && finite_bits(xr);
      const float xf = (float) xr;
      if (F32) {
        c[d] = abl::cell_coord_f32(xf, (float) lo[d], (float) inv_cell, dims[d]);
      } else {
        c[d] = abl::cell_coord((double) xr, lo[d], inv_cell, dims[d]);
      }
      m = fmaxf(m, fabsf(xf));
    }
    if (!finite) atomicExch(error, ABL_E_NONFINITE);
    int cell = (c[2] * ny + c[1]) * nx + c[0];
    cell_of[i] = cell;
    local_rank[i] = atomicAdd(&cell_count[cell], 1);
  }
  fold_amax(m, amax);
}

__global__ void k_bin_scatter(long n, const int *cell_of, const int *local_rank,
                              const int *cell_start, int *order) {
  long i = (long) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  bin_scatter_item(i, cell_of, local_rank, cell_start, order);
}

// One thread per cell: its run of slots sorted by agent id.
__global__ void k_cell_sort(long ncells, const int *cell_start, int *order) {
  long c = (long) blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  cell_sort_item(c, cell_start, order);
}

// Largest |coordinate| of a type that is not binned (query side only).
template <typename Real, int DIM>
__global__ void k_amax(const Real *pos, long n, float *amax, int *error) {
  long i = (long) blockIdx.x * blockDim.x + threadIdx.x;
  float m = 0.0f;
  if (i < n) {
    bool finite = true;
#pragma unroll
    for (int d = 0; d < DIM; d++) {
      double x = (double) pos[DIM * i + d];
      finite = finite && isfinite(x);
      m = fmaxf(m, fabsf((float) x));
    }
    if (!finite) atomicExch(error, ABL_E_NONFINITE);
  }
  fold_amax(m, amax);
}

__global__ void k_max2(const float *a, const float *b, float *out) {
  *out = fmaxf(*a, *b);
}

// sum() of a bool (1 byte) or int (4 byte) column.
__global__ void k_sum_int(const void *col, int bytes, long n, unsigned long long *out) {
  long i = (long) blockIdx.x * blockDim.x + threadIdx.x;
  long long v = 0;
  if (i < n) v = bytes == 1 ? (long long) ((const uint8_t *) col)[i] : ((const int *) col)[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v != 0) atomicAdd(out, (unsigned long long) v);
}

// sum() of floating-point members in ascending agent order (one thread).
__global__ void k_sum_seq(const void *col, int scalar, int comps, long n, double *out) {
  for (int c = 0; c < comps; c++) {
    if (scalar == 4) {
      float acc = 0.0f;
      for (long i = 0; i < n; i++) acc = acc + ((const float *) col)[comps * i + c];
      out[c] = acc;
    } else {
      double acc = 0.0;
      for (long i = 0; i < n; i++) acc = acc + ((const double *) col)[comps * i + c];
      out[c] = acc;
    }
  }
}

struct EqArgs {
  unsigned char value[24];
  int bytes, scalar, is_float;
};

// count(Type.member, value): element equality in the member's type.
__global__ void k_count_eq(const void *col, long n, const __grid_constant__ EqArgs a,
                           unsigned long long *out) {
  long i = (long) blockIdx.x * blockDim.x + threadIdx.x;
  int eq = 0;
  if (i < n) {
    const unsigned char *e = (const unsigned char *) col + (long) a.bytes * i;
    eq = 1;
    if (a.is_float && a.scalar == 8) {
      for (int c = 0; c < a.bytes / 8; c++)
        eq &= ((const double *) e)[c] == ((const double *) a.value)[c];
    } else if (a.is_float) {
      for (int c = 0; c < a.bytes / 4; c++)
        eq &= ((const float *) e)[c] == ((const float *) a.value)[c];
    } else if (a.bytes == 1) {
      eq = (e[0] != 0) == (a.value[0] != 0);
    } else {
      eq = *(const int *) e == *(const int *) a.value;
    }
  }
  unsigned m = __ballot_sync(0xffffffffu, eq);
  if ((threadIdx.x & 31) == 0 && m) atomicAdd(out, (unsigned long long) __popc(m));
}

template <typename Real, int DIM>
__global__ void k_gather(long n, const int *order, const Real *pos, float *posf,
                         const __grid_constant__ GatherArgs g) {
  long s = (long) blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  gather_item<Real, DIM>(s, order, pos, posf, g);
}

template <typename G, int AXIS>
__global__ void k_sep_count(long ncells, G geo, const int *src_off, int *dst_cnt) {
  const long c = (long) blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  sep_count_item<G, AXIS>(c, geo, src_off, dst_cnt);
}

// One thread per target cell with R = 1 (short lists: level 0).
template <typename G, int AXIS, bool LEVEL0>
__global__ void __launch_bounds__(kSepThreads)
k_sep_merge(long ncells, G geo, SepSrc S, const int *dst_off, int4 *dst_elem, int *dst_slot) {
  const long t = (long) blockIdx.x * kSepThreads + threadIdx.x;
  if (t >= ncells) return;
  sep_merge_item<G, AXIS, LEVEL0>(t, geo, S, dst_off, dst_elem, dst_slot);
}

// Level 0 of a single grid (R = 1), one thread per source slot: the three
// runs merged into cell t's list are the runs of cells t-1, t and t+1, so the
// slot's element goes to the lists of its own cell and of its x-neighbours.
// Its place in each is its index in its own run plus the number of smaller
// ids in the other two runs (binary searches over the short, id-sorted runs).
// The loads are independent, where a thread merging a cell's list waits on
// one load per element.  Writes the same lists as k_sep_merge<G, 0, true>.
template <typename G>
__global__ void k_sep_rows_by_slot(long n, G geo, const int *cell_start, const int *order,
                                   const float *posf, int dim, const int *cell_of,
                                   const int *dst_off, int4 *dst_elem) {
  const long e = (long) blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int id = __ldg(&order[e]);
  const int c = __ldg(&cell_of[id]);
  const CellPos P = cell_pos(geo, c);
  const int own = (int) e - __ldg(&cell_start[c]);
  const int4 v = make_int4(id, (int) e, __float_as_int(__ldg(&posf[dim * e])),
                           __float_as_int(__ldg(&posf[dim * e + 1])));
  const int x = P.x[0], nx = P.n[0];
#pragma unroll
  for (int d = -1; d <= 1; d++) {
    const int xt = x + d;
    if (xt < 0 || xt >= nx) continue;
    const int t = c + d;
    int rank = own;
#pragma unroll
    for (int k = -1; k <= 1; k++) {
      const int xu = xt + k;
      if (xu < 0 || xu >= nx || t + k == c) continue;
      const int b = __ldg(&cell_start[t + k]);
      int len = __ldg(&cell_start[t + k + 1]) - b, lo = 0;
      while (len > 0) {
        const int half = len >> 1;
        if (__ldg(&order[b + lo + half]) < id) {
          lo += half + 1;
          len -= half + 1;
        } else {
          len = half;
        }
      }
      rank += lo;
    }
    dst_elem[__ldg(&dst_off[t]) + rank] = v;
  }
}

// One warp per target cell with R = 1, the source ids staged in shared
// memory.
template <typename G, int AXIS, bool LEVEL0>
__global__ void __launch_bounds__(32 * kSepWarps)
k_sep_merge_warp(long ncells, G geo, SepSrc S, const int *dst_off, int4 *dst_elem,
                 int *dst_slot) {
  __shared__ int ids[kSepWarps][kSepStage];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long t = (long) blockIdx.x * kSepWarps + w;
  if (t >= ncells) return;  // uniform over the warp
  sep_merge_warp_item<G, AXIS, LEVEL0>(t, lane, geo, S, dst_off, dst_elem, dst_slot, ids[w]);
}

// One warp per target cell of a grid with R > 1.
template <typename G, int AXIS>
__global__ void __launch_bounds__(32 * kSepWarps)
k_sep_merge_large(long ncells, G geo, SepSrc S, const int *dst_off, int4 *dst_elem,
                  int *dst_slot) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long t = (long) blockIdx.x * kSepWarps + w;
  if (t >= ncells) return;
  sep_merge_large_item<G, AXIS>(t, lane, geo, S, dst_off, dst_elem, dst_slot);
}


// Intermediate levels of the separable list build (dim - 1 of them).
struct SepLevels {
  int *off[2] = {nullptr, nullptr};
  int4 *elem[2] = {nullptr, nullptr};
};

// --------------------------------------------------------------- state

struct TypeState {
  const abl_agent_desc *d = nullptr;
  long n = 0;
  long cap = 0;            // agents the column buffers can hold
  bool dynamic = false;    // some step function removes or adds agents of this type
  bool uploaded = false;
  bool reserved_resize = false;  // abl_reserve resized the buffers; abl_commit re-prepares
  void *cols[2][ABL_MAX_MEMBERS] = {};
  int cur = 0;
  float *amax = nullptr;  // this type's largest |coordinate| (device)

  // binning (near types only)
  bool is_near = false;
  bool ordered = false;     // whole neighbourhood lists (list depth 2)
  bool rows = false;        // row lists (list depth 1)
  bool dirty = true;
  // Only gathered non-position members changed (positions of this type are
  // never written): the binning stands, the slot-ordered copies are stale.
  bool regather = false;
  long bin_id = 0;           // serial number of the last full binning
  int R = 1;
  int nx = 1, ny = 1, nz = 1;
  long ncells = 1;
  double lo[3] = {0, 0, 0};
  double inv_cell = 1.0;
  uint32_t gather_mask = 0;
  int *cell_count = nullptr, *cell_start = nullptr, *local_rank = nullptr, *cell_of = nullptr;
  int *order = nullptr;
  float *posf = nullptr;
  void *gcols[ABL_MAX_MEMBERS] = {};
  // Mixed precision: members summed in FP32 get slot-ordered float copies,
  // and position offsets need the position's low part.
  uint32_t gather_f32_mask = 0;
  bool gather_pos_lo = false;
  void *fcols[ABL_MAX_MEMBERS] = {};
  float *poslo = nullptr;
  int *nb_cnt = nullptr, *nb_off = nullptr, *nb_list = nullptr;
  SepLevels sep;
  ScanPlan cell_scan, nb_scan;
  std::vector<void *> bin_allocs;  // freed when the type is re-uploaded
};

// Neighbour lists a near step's grid gets: 0 none (presorted loops sort
// each agent's neighbours from the cells' runs), 1 row lists (2D presorted
// loops merge the rows above, at and below on the fly), 2 whole
// neighbourhood lists (every other ordered loop).  By default presorted loops
// whose agents are the binned ones (threads visit agents cell by cell, so a
// warp reads few lists in lockstep) use row lists in 2D and whole lists in
// 3D; loops over another type sort the cells' runs per agent.  `mode`
// (ABL_NEAR_*) forces one of them.
int list_depth(const abl_step_desc &sd, const abl_agent_desc &d, int mode) {
  if (!sd.ordered) return 0;
  if (!sd.presorted) return 2;
  switch (mode) {
    case ABL_NEAR_RUNS: return 0;
    case ABL_NEAR_ROWS: return d.dim == 2 ? 1 : 0;
    case ABL_NEAR_BLOCK: return d.dim == 2 ? 1 : 0;
    case ABL_NEAR_LISTS: return 2;
    default: break;
  }
  if (sd.agent_type != sd.near_type) return 0;
  return d.dim == 2 ? 1 : 2;
}

// Block lists (abl_device.cuh, gather_block) serve 2D row-list loops whose
// agents are the binned ones, unless the mode asks for per-agent rows.
bool block_lists_wanted(const abl_step_desc &sd, int depth, int mode) {
  return depth == 1 && sd.agent_type == sd.near_type
      && (mode == ABL_NEAR_AUTO || mode == ABL_NEAR_BLOCK);
}

size_t member_bytes(const abl_member_desc &m) {
  return (size_t) m.components * m.scalar_bytes;
}

}  // namespace

// Per step function buffers for runtime removal and addition.
struct StepState {
  uint8_t *removed = nullptr;               // parent capacity
  uint8_t *child_flag = nullptr;            // parent capacity
  void *child_cols[ABL_MAX_MEMBERS] = {};   // added type's members, parent capacity
  int *keep = nullptr, *keep_pos = nullptr; // parent capacity (+1)
  int *child = nullptr, *child_pos = nullptr;
  ScanPlan keep_scan, child_scan;
  long parent_cap = 0;
  // Neighbour lists kept across timesteps (static positions): per agent of
  // the step's type the indices of its in-radius neighbours, ascending (int16
  // offsets from the agent's own index when they all fit), and the agents'
  // float positions by index.  Built for binning `nc_bin` of the step's grid
  // (-1: none); nc_off null with nc_bin set means they did not fit.
  int *nc_off = nullptr;
  void *nc_list = nullptr;  // nc_wide or nc_short
  bool nc_narrow = false;
  float *nc_posf = nullptr;
  long nc_bin = -1;
  double nc_radius = 0.0;
  // Buffers kept from one build to the next (a rebuild after an upload
  // reuses them, so graphs captured earlier stay valid).
  int *nc_count = nullptr, *nc_span = nullptr, *nc_wide = nullptr;
  short *nc_short = nullptr;
  ScanPlan nc_scan;
  long nc_n = 0, nc_wide_cap = 0, nc_short_cap = 0;
  std::vector<void *> nc_allocs;
};

struct abl_ctx {
  const abl_model_desc *model = nullptr;
  std::vector<unsigned char> globals;
  cudaStream_t stream = nullptr;
  std::vector<TypeState> types;
  size_t budget = 0, used = 0;
  std::vector<void *> allocations;
  std::vector<size_t> sizes;
  int *error = nullptr;
  float *amax_pair = nullptr;  // per step: max of query and neighbour amax
  int *error_host = nullptr;   // pinned copy of `error` read by check_error
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_exec = 0.0;
  long launches = 0, last_launches = 0;
  // Captured two-timestep graphs, keyed by the buffer parity and binning
  // state they start from (kernel arguments depend on both).
  struct Graph {
    std::vector<int> key;      // state (parities, dirty flags) and timesteps captured
    std::vector<int> end_key;  // state after the captured timesteps
    int steps = 0;
    cudaGraphExec_t exec = nullptr;
    long launches = 0;
  };
  std::vector<Graph> graphs;
  // An eager timestep has run since the graphs were dropped (allocations and
  // binnings settled), so timesteps may be captured.
  bool warm = false;
  bool prepared = false;
  // One uniform grid per (neighbour type, cell size): every near loop bins
  // its neighbour type with cells just wider than its own radius.
  std::vector<TypeState> grids;
  std::vector<int> grid_type;  // grid -> agent type
  std::vector<int> step_grid;  // step function -> grid (-1: no near loop)
  std::vector<StepState> step_state;
  std::vector<void *> step_allocs;
  uint64_t seed = 0;
  long timestep = 0;
  cudaEvent_t ts0 = nullptr, ts1 = nullptr;
  double last_timestep = 0.0;
  int seq_error = 0;  // first error of a builtin called by the sequential step
  std::string log;
  int *d_pair = nullptr;   // two ints read back after compaction scans
  double *d_red = nullptr; // reduction results
  // Optional per-step-function kernel timing (eager timesteps only).
  bool profile = false;
  // Presorted near steps: hand each block's agents to threads by neighbour
  // count; neighbours held per agent in shared memory with and without
  // neighbourhood lists (4 and 8 bytes each).
  int balance = 1;
  int list_cap = ABL_LIST_CAP;
  int runs_cap = 40;
  int near_mode = ABL_NEAR_AUTO;
  // Entries of a thread block's shared-memory neighbourhood lists (ABL_NEAR_BLOCK).
  int block_cap = 2048;
  bool near_cache = true;
  long bin_serial = 0;
  // Step kernels skip stores of members that never change (both buffers
  // hold them since the upload).
  bool skip_stores = true;
  // Sequential random numbers (abl_set_serial_random): the xorshift128+
  // state on the device, and agent indices 0..n-1 for one-agent launches.
  unsigned long long *serial_rng = nullptr;
  int *serial_iota = nullptr;
  long serial_iota_n = 0;
  std::vector<std::vector<std::pair<cudaEvent_t, cudaEvent_t>>> prof_pending;
  std::vector<double> prof_seconds;
  std::vector<long> prof_launches;
};

namespace {

// A named range on the host timeline (NVTX): binning, list builds, each step
// function's launch, compaction, uploads, downloads and reductions show up
// as phases in profilers.  Without a tool attached it costs a call.
struct Phase {
  explicit Phase(const char *name) { nvtxRangePushA(name); }
  ~Phase() { nvtxRangePop(); }
};

// Device memory comes from the device's stream-ordered pool (cudaMallocAsync
// on the context's stream).  cudaMalloc and cudaFree synchronise the whole
// device, so contexts created and destroyed while others run (the job
// server) would stall every running simulation; pool allocations and frees
// wait only for the context's own stream.  The pool keeps freed memory for
// reuse instead of returning it at each synchronisation.
void keep_pool_memory() {
  static std::once_flag once;
  std::call_once(once, [] {
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t keep = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  });
}

// Pinned words that check_error reads the device error word into, one per
// context, from one pinned block allocated once: pinned allocations, like
// device ones, synchronise the device.
constexpr int kErrorSlots = 4096;
std::mutex error_slot_mu;
int *error_slots = nullptr;
std::vector<int> free_error_slots;

cudaError_t take_error_slot(int **slot) {
  std::lock_guard<std::mutex> lock(error_slot_mu);
  if (!error_slots) {
    cudaError_t e = cudaHostAlloc((void **) &error_slots, sizeof(int) * kErrorSlots,
                                  cudaHostAllocDefault);
    if (e != cudaSuccess) {
      error_slots = nullptr;
      return e;
    }
    for (int k = kErrorSlots - 1; k >= 0; k--) free_error_slots.push_back(k);
  }
  if (free_error_slots.empty()) {
    *slot = nullptr;  // check_error then reads the word with a plain copy
    return cudaSuccess;
  }
  *slot = error_slots + free_error_slots.back();
  free_error_slots.pop_back();
  return cudaSuccess;
}

void release_error_slot(int *slot) {
  if (!slot) return;
  std::lock_guard<std::mutex> lock(error_slot_mu);
  free_error_slots.push_back((int) (slot - error_slots));
}

int dev_alloc(abl_ctx *ctx, void **p, size_t bytes, std::vector<void *> *owner = nullptr) {
  if (bytes == 0) bytes = 16;
  bytes = (bytes + 255) & ~(size_t) 255;
  if (ctx->budget && ctx->used + bytes > ctx->budget) return ABL_E_BUDGET;
  keep_pool_memory();
  // The block is in use on any stream once the context's stream has reached
  // the allocation (host copies address it right away).
  cudaError_t e = cudaMallocAsync(p, bytes, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    std::fprintf(stderr, "openabl-cuda: cudaMallocAsync(%zu) failed: %s\n", bytes,
                 cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? ABL_E_BUDGET : ABL_E_CUDA;
  }
  ctx->used += bytes;
  ctx->allocations.push_back(*p);
  ctx->sizes.push_back(bytes);
  if (owner) owner->push_back(*p);
  return ABL_OK;
}

void dev_free(abl_ctx *ctx, void *p) {
  for (size_t k = 0; k < ctx->allocations.size(); k++) {
    if (ctx->allocations[k] == p) {
      cudaFreeAsync(p, ctx->stream);
      ctx->used -= ctx->sizes[k];
      ctx->allocations.erase(ctx->allocations.begin() + k);
      ctx->sizes.erase(ctx->sizes.begin() + k);
      return;
    }
  }
}

template <typename T>
int dev_alloc_t(abl_ctx *ctx, T **p, size_t count, std::vector<void *> *owner = nullptr) {
  void *v = nullptr;
  int r = dev_alloc(ctx, &v, count * sizeof(T), owner);
  *p = (T *) v;
  return r;
}

int scan_plan(abl_ctx *ctx, ScanPlan &p, long m, std::vector<void *> *owner) {
  p.levels.clear();
  long len = m;
  for (;;) {
    ScanLevel L;
    L.m = len;
    L.nb = std::max<long>(1, (len + kScanBlock - 1) / kScanBlock);
    ABL_TRY(dev_alloc_t(ctx, &L.incl, std::max<long>(len, 1), owner));
    ABL_TRY(dev_alloc_t(ctx, &L.sums, L.nb, owner));
    ABL_TRY(dev_alloc_t(ctx, &L.offs, L.nb + 1, owner));
    p.levels.push_back(L);
    if (L.nb == 1) break;
    len = L.nb;
  }
  return ABL_OK;
}

void scan_level(abl_ctx *ctx, const ScanPlan &p, size_t l, const int *in, int *out) {
  const ScanLevel &L = p.levels[l];
  cudaStream_t s = ctx->stream;
  if (L.nb == 1) {
    k_scan_single<<<1, kScanBlock / 4, 0, s>>>(in, out, L.m);
    ctx->launches++;
    return;
  }
  k_scan_blocks<<<L.nb, kScanBlock / 4, 0, s>>>(in, L.incl, L.m, L.sums);
  ctx->launches++;
  if (L.nb <= kScanBlock) {
    k_scan_finish_sums<<<(L.m + 255) / 256, 256, 0, s>>>(L.incl, out, L.m, L.sums);
    ctx->launches++;
    return;
  }
  scan_level(ctx, p, l + 1, L.sums, L.offs);
  k_scan_finish<<<(L.m + 1 + 255) / 256, 256, 0, s>>>(L.incl, out, L.m, L.offs);
  ctx->launches++;
}

// Exclusive scan of `in` (m ints) into `out` (m + 1 ints, out[m] = total).
void scan_run(abl_ctx *ctx, const ScanPlan &p, const int *in, int *out) {
  scan_level(ctx, p, 0, in, out);
}


inline long blocks_for(long n, int block) { return std::max<long>(1, (n + block - 1) / block); }

const abl_member_desc &pos_member(const TypeState &t) {
  return t.d->members[t.d->position_member];
}

bool pos_is_double(const TypeState &t) { return pos_member(t).scalar_bytes == 8; }

// Largest near radius over the step functions that iterate type `ti`.
double max_radius_for(const abl_ctx *ctx, int ti) {
  double r = 0.0;
  for (int k = 0; k < ctx->model->num_steps; k++) {
    const abl_step_desc &sd = ctx->model->steps[k];
    if (sd.near_type == ti && sd.radius) r = std::max(r, sd.radius(ctx->globals.data()));
  }
  return r;
}

void free_bins(abl_ctx *ctx, TypeState &t) {
  for (void *p : t.bin_allocs) dev_free(ctx, p);
  t.bin_allocs.clear();
  t.cell_scan.levels.clear();
  t.nb_scan.levels.clear();
  t.cell_count = t.cell_start = t.local_rank = t.cell_of = t.order = nullptr;
  t.nb_cnt = t.nb_off = t.nb_list = nullptr;
  t.sep = SepLevels();
  t.posf = nullptr;
  for (auto &g : t.gcols) g = nullptr;
  for (auto &f : t.fcols) f = nullptr;
  t.poslo = nullptr;
}

// Sizes one grid per (neighbour type, cell size) -- the cells of a near
// loop's grid are just wider than the loop's radius, so each loop scans ~9
// (2D) or ~27 (3D) cells' worth of its radius, whatever the environment
// granularity (src/AnalysisVisitor.cpp:1378-1399, which only partitions
// space and does not change results) -- and allocates the binning buffers.
void nc_free_all(abl_ctx *ctx, StepState &st);

int prepare(abl_ctx *ctx) {
  const abl_model_desc *m = ctx->model;
  const void *G = ctx->globals.data();
  double emin[3] = {0, 0, 0}, emax[3] = {0, 0, 0};
  if (m->env_bounds) m->env_bounds(G, emin, emax);
  for (int ti = 0; ti < m->num_agent_types; ti++) {
    TypeState &t = ctx->types[ti];
    if (!t.amax) ABL_TRY(dev_alloc_t(ctx, &t.amax, 1));
  }
  for (TypeState &g : ctx->grids) free_bins(ctx, g);
  ctx->grids.clear();
  ctx->grid_type.clear();
  ctx->step_grid.assign(m->num_steps, -1);
  std::vector<double> grid_cell;
  for (int k = 0; k < m->num_steps; k++) {
    const abl_step_desc &sd = m->steps[k];
    if (sd.near_type < 0) continue;
    int ti = sd.near_type;
    if (ctx->types[ti].d->position_member < 0) return ABL_E_UNSUPPORTED;
    double r = sd.radius ? sd.radius(G) : 0.0;
    if (!(r > 0.0) || !std::isfinite(r)) {
      // A radius that is not a positive number: one cell per axis unit of the
      // granularity (every candidate then takes the exact test).
      r = m->granularity ? m->granularity(G) : max_radius_for(ctx, ti);
    }
    if (!(r > 0.0) || !std::isfinite(r)) return ABL_E_INVALID;
    // Cells slightly wider than the radius: a pair that passes the
    // float-rounded radius test lies within one cell width (see
    // abl_device.cuh), with room for rounding in the cell computation.
    double cell = r * (1.0 + 1.0 / 1024.0);
    int gi = -1;
    for (size_t q = 0; q < ctx->grids.size(); q++) {
      if (ctx->grid_type[q] == ti && grid_cell[q] == cell) gi = (int) q;
    }
    if (gi < 0) {
      gi = (int) ctx->grids.size();
      ctx->grids.emplace_back();
      ctx->grid_type.push_back(ti);
      grid_cell.push_back(cell);
      TypeState &g = ctx->grids.back();
      g.d = ctx->types[ti].d;
      g.is_near = true;
    }
    TypeState &g = ctx->grids[gi];
    const int depth = list_depth(sd, *g.d, ctx->near_mode);
    g.ordered = g.ordered || depth == 2;
    g.rows = g.rows || depth == 1;
    g.gather_mask |= sd.near_members;
    g.gather_f32_mask |= sd.near_members_f32;
    g.gather_pos_lo = g.gather_pos_lo || sd.near_pos_lo;
    ctx->step_grid[k] = gi;
  }
  for (size_t gi = 0; gi < ctx->grids.size(); gi++) {
    TypeState &g = ctx->grids[gi];
    const TypeState &t = ctx->types[ctx->grid_type[gi]];
    int dim = g.d->dim;
    double cell = grid_cell[gi];
    // At most ~2 cells per agent: scans and list building cost per cell, and
    // finer cells than that stop reducing the candidates worth visiting.
    {
      double max_cells = std::max(4096.0, 2.0 * (double) std::max(t.n, t.cap));
      double vol = 1.0;
      for (int d = 0; d < dim; d++) vol *= std::max(emax[d] - emin[d], cell);
      double cells = vol / std::pow(cell, dim);
      if (cells > max_cells && std::isfinite(vol)) cell = std::pow(vol / max_cells, 1.0 / dim);
    }
    g.inv_cell = 1.0 / cell;
    g.R = 1;
    int dims[3] = {1, 1, 1};
    for (int d = 0; d < 3; d++) {
      if (d < dim) {
        double ext = emax[d] - emin[d];
        if (!(ext >= 0.0) || !std::isfinite(ext)) return ABL_E_INVALID;
        double k = std::floor(ext * g.inv_cell) + 1.0;
        if (k > 1 << 24) return ABL_E_UNSUPPORTED;
        dims[d] = (int) k;
        g.lo[d] = emin[d];
      } else {
        g.lo[d] = 0.0;
      }
    }
    g.nx = dims[0];
    g.ny = dims[1];
    g.nz = dims[2];
    g.ncells = (long) g.nx * g.ny * g.nz;
    if (g.ncells > (1L << 30)) return ABL_E_UNSUPPORTED;
    g.n = t.n;
    g.cap = t.cap;
    long n = std::max<long>(std::max(t.n, t.cap), 1);
    auto *own = &g.bin_allocs;
    ABL_TRY(dev_alloc_t(ctx, &g.amax, 1, own));
    ABL_TRY(dev_alloc_t(ctx, &g.cell_count, g.ncells, own));
    ABL_TRY(dev_alloc_t(ctx, &g.cell_start, g.ncells + 1, own));
    ABL_TRY(dev_alloc_t(ctx, &g.local_rank, n, own));
    ABL_TRY(dev_alloc_t(ctx, &g.cell_of, n, own));
    ABL_TRY(dev_alloc_t(ctx, &g.order, n, own));
    ABL_TRY(dev_alloc_t(ctx, &g.posf, n * dim, own));
    ABL_TRY(scan_plan(ctx, g.cell_scan, g.ncells, own));
    for (int k = 0; k < g.d->num_members; k++) {
      if (g.gather_mask & (1u << k)) {
        void *p = nullptr;
        ABL_TRY(dev_alloc(ctx, &p, member_bytes(g.d->members[k]) * n, own));
        g.gcols[k] = p;
      }
      if (g.gather_f32_mask & (1u << k)) {
        void *p = nullptr;
        ABL_TRY(dev_alloc(ctx, &p, sizeof(float) * g.d->members[k].components * n, own));
        g.fcols[k] = p;
      }
    }
    if (g.gather_pos_lo) ABL_TRY(dev_alloc_t(ctx, &g.poslo, n * dim, own));
    if (g.ordered || g.rows) {
      long span = 2 * g.R + 1, level = n;
      const int inter = g.ordered ? dim - 1 : 1;  // levels kept as (id, slot) lists
      for (int a = 0; a < inter; a++) {
        level *= span;
        ABL_TRY(dev_alloc_t(ctx, &g.sep.off[a], g.ncells + 1, own));
        ABL_TRY(dev_alloc_t(ctx, &g.sep.elem[a], level, own));
      }
      // List offsets are 32-bit.
      if (level * (g.ordered ? span : 1) > (long) INT32_MAX) return ABL_E_UNSUPPORTED;
      ABL_TRY(dev_alloc_t(ctx, &g.nb_cnt, g.ncells, own));
      ABL_TRY(scan_plan(ctx, g.nb_scan, g.ncells, own));
      if (g.ordered) {
        ABL_TRY(dev_alloc_t(ctx, &g.nb_off, g.ncells + 1, own));
        ABL_TRY(dev_alloc_t(ctx, &g.nb_list, level * span, own));
      }
    }
    g.dirty = true;
  }
  if (!ctx->amax_pair) ABL_TRY(dev_alloc_t(ctx, &ctx->amax_pair, 1));
  if (!ctx->d_pair) ABL_TRY(dev_alloc_t(ctx, &ctx->d_pair, 2));
  // Buffers of step functions that remove or add agents, sized by the
  // capacity of the step's own type (one flag / one child per agent).
  for (void *p : ctx->step_allocs) dev_free(ctx, p);
  ctx->step_allocs.clear();
  for (StepState &st : ctx->step_state) nc_free_all(ctx, st);
  ctx->step_state.assign(m->num_steps, StepState());
  for (int k = 0; k < m->num_steps; k++) {
    const abl_step_desc &sd = m->steps[k];
    if (!sd.uses_remove && sd.add_type < 0) continue;
    StepState &st = ctx->step_state[k];
    const TypeState &pt = ctx->types[sd.agent_type];
    long pc = std::max<long>(std::max(pt.cap, pt.n), 1);
    st.parent_cap = pc;
    auto *own = &ctx->step_allocs;
    ABL_TRY(dev_alloc_t(ctx, &st.removed, pc, own));
    ABL_TRY(dev_alloc_t(ctx, &st.child_flag, pc, own));
    ABL_TRY(dev_alloc_t(ctx, &st.keep, pc, own));
    ABL_TRY(dev_alloc_t(ctx, &st.keep_pos, pc + 1, own));
    ABL_TRY(dev_alloc_t(ctx, &st.child, pc, own));
    ABL_TRY(dev_alloc_t(ctx, &st.child_pos, pc + 1, own));
    ABL_TRY(scan_plan(ctx, st.keep_scan, pc, own));
    ABL_TRY(scan_plan(ctx, st.child_scan, pc, own));
    if (sd.add_type >= 0) {
      const abl_agent_desc &ad = m->agents[sd.add_type];
      for (int j = 0; j < ad.num_members; j++) {
        void *p = nullptr;
        ABL_TRY(dev_alloc(ctx, &p, member_bytes(ad.members[j]) * pc, own));
        st.child_cols[j] = p;
      }
    }
  }
  ctx->prepared = true;
  return ABL_OK;
}

// ------------------------------------------------- removal and addition

// keep[i] = 1 unless agent i removed itself; child[i] = 1 when it added one.
__global__ void k_flags(long n, const uint8_t *removed, const uint8_t *child_flag, int *keep,
                        int *child) {
  long i = (long) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  keep[i] = removed ? (removed[i] ? 0 : 1) : 1;
  child[i] = child_flag ? (child_flag[i] ? 1 : 0) : 0;
}

__global__ void k_read_totals(const int *a, long na, const int *b, long nb, int *out) {
  out[0] = a ? a[na] : 0;
  out[1] = b ? b[nb] : 0;
}

struct MoveArgs {
  int nmem;
  const void *src[ABL_MAX_MEMBERS];
  void *dst[ABL_MAX_MEMBERS];
  int bytes[ABL_MAX_MEMBERS];
};

__device__ inline void copy_elem(const void *src, void *dst, long si, long di, int b) {
  if ((b & 7) == 0) {
    const uint64_t *s = (const uint64_t *) src + (b / 8) * si;
    uint64_t *d = (uint64_t *) dst + (b / 8) * di;
    for (int w = 0; w < b / 8; w++) d[w] = s[w];
  } else if ((b & 3) == 0) {
    const uint32_t *s = (const uint32_t *) src + (b / 4) * si;
    uint32_t *d = (uint32_t *) dst + (b / 4) * di;
    for (int w = 0; w < b / 4; w++) d[w] = s[w];
  } else {
    const uint8_t *s = (const uint8_t *) src + b * si;
    uint8_t *d = (uint8_t *) dst + b * di;
    for (int w = 0; w < b; w++) d[w] = s[w];
  }
}

// Stable compaction: element i moves to base + pos[i] when flag[i] is set.
__global__ void k_scatter_flagged(long n, const int *flag, const int *pos, long base,
                                  const __grid_constant__ MoveArgs a) {
  long i = (long) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !flag[i]) return;
  long di = base + pos[i];
  for (int k = 0; k < a.nmem; k++) copy_elem(a.src[k], a.dst[k], i, di, a.bytes[k]);
}

// Grows a type's column buffers to hold `need` agents, keeping the first n
// agents of both buffers.
int grow_type(abl_ctx *ctx, TypeState &t, long need) {
  long cap = std::max(need, 2 * std::max<long>(t.cap, 1));
  for (int b = 0; b < 2; b++) {
    for (int k = 0; k < t.d->num_members; k++) {
      void *p = nullptr;
      size_t mb = member_bytes(t.d->members[k]);
      ABL_TRY(dev_alloc(ctx, &p, mb * cap));
      if (t.n > 0) {
        ABL_CUDA_TRY(cudaMemcpyAsync(p, t.cols[b][k], mb * t.n, cudaMemcpyDeviceToDevice,
                                     ctx->stream));
      }
      ABL_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
      dev_free(ctx, t.cols[b][k]);
      t.cols[b][k] = p;
    }
  }
  t.cap = cap;
  return ABL_OK;
}

MoveArgs move_args(const abl_agent_desc &d, void *const *src, void *const *dst) {
  MoveArgs a;
  std::memset(&a, 0, sizeof a);
  a.nmem = d.num_members;
  for (int k = 0; k < d.num_members; k++) {
    a.src[k] = src[k];
    a.dst[k] = dst[k];
    a.bytes[k] = (int) member_bytes(d.members[k]);
  }
  return a;
}

void mark_dirty(abl_ctx *ctx, int ti);


// After a step function that removes or adds agents: stable compaction of
// the survivors, then the children appended in parent order.  The step's
// result is in the buffer it wrote (cols[1 - cur]).  Returns with `regrow`
// set when a type had to grow (the binning buffers are then resized before
// the next binning).
int apply_population_changes(abl_ctx *ctx, int k, bool &regrow) {
  const abl_step_desc &sd = ctx->model->steps[k];
  StepState &st = ctx->step_state[k];
  TypeState &t = ctx->types[sd.agent_type];
  cudaStream_t s = ctx->stream;
  const int B = 256;
  long n = t.n;
  long nb = blocks_for(n, B);
  bool self_add = sd.add_type == sd.agent_type;
  k_flags<<<nb, B, 0, s>>>(n, sd.uses_remove ? st.removed : nullptr,
                           sd.add_type >= 0 ? st.child_flag : nullptr, st.keep, st.child);
  ctx->launches++;
  // Only the scans a step needs: survivors when it removes, children when
  // it adds.
  const bool scan_keep = sd.uses_remove, scan_child = sd.add_type >= 0;
  if (scan_keep) scan_run(ctx, st.keep_scan, st.keep, st.keep_pos);
  if (scan_child) scan_run(ctx, st.child_scan, st.child, st.child_pos);
  k_read_totals<<<1, 1, 0, s>>>(scan_keep ? st.keep_pos : nullptr, n,
                                scan_child ? st.child_pos : nullptr, n, ctx->d_pair);
  ctx->launches++;
  int tot[2] = {0, 0};
  ABL_CUDA_TRY(cudaMemcpyAsync(tot, ctx->d_pair, sizeof tot, cudaMemcpyDeviceToHost, s));
  ABL_CUDA_TRY(cudaStreamSynchronize(s));
  long survivors = scan_keep ? tot[0] : n, children = scan_child ? tot[1] : 0;
  if (!sd.uses_remove && self_add) {
    // Nobody left: `out` becomes the current buffer as it is, and the
    // children follow its n agents.  (The double buffer's content does not
    // matter here: with runtime add/remove, step kernels start `out` as a
    // copy of `in`.)
    t.cur = 1 - t.cur;
    if (children > 0) {
      long need = n + children;
      if (need > t.cap) {
        ABL_TRY(grow_type(ctx, t, need));
        regrow = true;
      }
      MoveArgs c = move_args(*t.d, st.child_cols, t.cols[t.cur]);
      k_scatter_flagged<<<nb, B, 0, s>>>(n, st.child, st.child_pos, n, c);
      ctx->launches++;
      t.n = need;
    }
  } else if (sd.uses_remove) {
    long need = survivors + (self_add ? children : 0);
    // `out` holds the step's result; compact it into the other buffer.
    if (need > t.cap) {
      ABL_TRY(grow_type(ctx, t, need));
      regrow = true;
    }
    MoveArgs a = move_args(*t.d, t.cols[1 - t.cur], t.cols[t.cur]);
    k_scatter_flagged<<<nb, B, 0, s>>>(n, st.keep, st.keep_pos, 0, a);
    ctx->launches++;
    if (self_add && children > 0) {
      MoveArgs c = move_args(*t.d, st.child_cols, t.cols[t.cur]);
      k_scatter_flagged<<<nb, B, 0, s>>>(n, st.child, st.child_pos, survivors, c);
      ctx->launches++;
    }
    t.n = need;  // result now in cols[cur]
  } else {
    t.cur = 1 - t.cur;
  }
  if (sd.add_type >= 0 && !self_add && children > 0) {
    TypeState &t2 = ctx->types[sd.add_type];
    long need = t2.n + children;
    if (need > t2.cap) {
      ABL_TRY(grow_type(ctx, t2, need));
      regrow = true;
    }
    MoveArgs c = move_args(*t2.d, st.child_cols, t2.cols[t2.cur]);
    k_scatter_flagged<<<nb, B, 0, s>>>(n, st.child, st.child_pos, t2.n, c);
    ctx->launches++;
    t2.n = need;
    mark_dirty(ctx, sd.add_type);
  }
  mark_dirty(ctx, sd.agent_type);
  return ABL_OK;
}

// Builds the first `levels` axes of a binned grid's lists: the row lists
// (levels 1) or, with levels == dim, the whole neighbourhood lists (nb_off,
// nb_list).
template <typename G>
void build_lists(abl_ctx *ctx, const G &geo, int dim, int levels, int Rmax, long ncells,
                 const int *cell_start, const int *order, const float *posf,
                 const SepLevels &L, int *cnt, const ScanPlan &scan, int *nb_off, int *nb_list,
                 long nslots = 0, const int *cell_of = nullptr) {
  cudaStream_t s = ctx->stream;
  const int B = 256;
  SepSrc src{cell_start, order, posf, dim, nullptr};
  const long cb = blocks_for(ncells, B), lb = blocks_for(ncells, kSepWarps);
  for (int a = 0; a < levels; a++) {
    const bool last = a == dim - 1;
    int *off = last ? nb_off : L.off[a];
    int4 *de = last ? nullptr : L.elem[a];
    int *ds = last ? nb_list : nullptr;
    if (a == 0) k_sep_count<G, 0><<<cb, B, 0, s>>>(ncells, geo, src.off, cnt);
    else if (a == 1) k_sep_count<G, 1><<<cb, B, 0, s>>>(ncells, geo, src.off, cnt);
    else k_sep_count<G, 2><<<cb, B, 0, s>>>(ncells, geo, src.off, cnt);
    ctx->launches++;
    scan_run(ctx, scan, cnt, off);
    if (a == 0 && cell_of && de && Rmax == 1) {
      // A single grid's row lists: one thread per slot.
      k_sep_rows_by_slot<G><<<blocks_for(nslots, B), B, 0, s>>>(nslots, geo, cell_start, order,
                                                               posf, dim, cell_of, off, de);
    } else if (a == 0) {
      // Level 0 merges a few agents per cell: one thread per cell.  The
      // later levels' lists are 3 and 9 times longer: one warp per cell.
      k_sep_merge<G, 0, true><<<blocks_for(ncells, kSepThreads), kSepThreads, 0, s>>>(
          ncells, geo, src, off, de, ds);
      if (Rmax > 1) k_sep_merge_large<G, 0><<<lb, 32 * kSepWarps, 0, s>>>(ncells, geo, src, off, de, ds);
    } else if (a == 1) {
      k_sep_merge_warp<G, 1, false><<<lb, 32 * kSepWarps, 0, s>>>(ncells, geo, src, off, de, ds);
      if (Rmax > 1) k_sep_merge_large<G, 1><<<lb, 32 * kSepWarps, 0, s>>>(ncells, geo, src, off, de, ds);
    } else {
      k_sep_merge_warp<G, 2, false><<<lb, 32 * kSepWarps, 0, s>>>(ncells, geo, src, off, de, ds);
      if (Rmax > 1) k_sep_merge_large<G, 2><<<lb, 32 * kSepWarps, 0, s>>>(ncells, geo, src, off, de, ds);
    }
    ctx->launches += Rmax > 1 ? 2 : 1;
    if (!last) src = SepSrc{L.off[a], nullptr, nullptr, dim, L.elem[a]};
  }
}

// Slot-ordered copies of the gathered members (and, with_pos, the float
// positions); without with_pos the position member itself is skipped too.
// Mixed precision: float copies of members summed in FP32, and the
// position's low part (float) (pos - (double) posf), in slot order.
struct GatherF32Args {
  int nmem;
  const double *src[ABL_MAX_MEMBERS];
  float *dst[ABL_MAX_MEMBERS];
  int comps[ABL_MAX_MEMBERS];
};

template <int DIM>
__global__ void k_gather_f32(long n, const int *order, const double *pos, const float *posf,
                             float *poslo, const __grid_constant__ GatherF32Args g) {
  long s = (long) blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  long i = order[s];
  if (poslo) {
#pragma unroll
    for (int d = 0; d < DIM; d++)
      poslo[DIM * s + d] = (float) (pos[DIM * i + d] - (double) posf[DIM * s + d]);
  }
  for (int k = 0; k < g.nmem; k++) {
    const int c = g.comps[k];
    for (int j = 0; j < c; j++) g.dst[k][c * s + j] = (float) g.src[k][c * i + j];
  }
}

void launch_gather_f32(abl_ctx *ctx, TypeState &t, int dim, bool with_pos) {
  GatherF32Args g;
  std::memset(&g, 0, sizeof g);
  for (int k = 0; k < t.d->num_members; k++) {
    if (!(t.gather_f32_mask & (1u << k))) continue;
    if (!with_pos && k == t.d->position_member) continue;
    g.src[g.nmem] = (const double *) t.cols[t.cur][k];
    g.dst[g.nmem] = (float *) t.fcols[k];
    g.comps[g.nmem] = t.d->members[k].components;
    g.nmem++;
  }
  float *poslo = with_pos && t.gather_pos_lo ? t.poslo : nullptr;
  if (!poslo && g.nmem == 0) return;
  const double *pos = (const double *) t.cols[t.cur][t.d->position_member];
  const int B = 256;
  long nb = blocks_for(t.n, B);
  if (dim == 2) k_gather_f32<2><<<nb, B, 0, ctx->stream>>>(t.n, t.order, pos, t.posf, poslo, g);
  else k_gather_f32<3><<<nb, B, 0, ctx->stream>>>(t.n, t.order, pos, t.posf, poslo, g);
  ctx->launches++;
}

template <typename Real>
void launch_gather(abl_ctx *ctx, TypeState &t, int dim, bool with_pos) {
  cudaStream_t s = ctx->stream;
  const int B = 256;
  long nb = blocks_for(t.n, B);
  const Real *pos = (const Real *) t.cols[t.cur][t.d->position_member];
  GatherArgs g;
  std::memset(&g, 0, sizeof g);
  g.pos16 = -1;
  for (int k = 0; k < t.d->num_members; k++) {
    if (!(t.gather_mask & (1u << k))) continue;
    if (!with_pos && k == t.d->position_member) continue;
    if (k == t.d->position_member) g.pos16 = g.nmem;
    g.src[g.nmem] = t.cols[t.cur][k];
    g.dst[g.nmem] = t.gcols[k];
    g.bytes[g.nmem] = (int) member_bytes(t.d->members[k]);
    g.nmem++;
  }
  g.all16 = g.nmem > 0 && g.nmem <= 4;
  for (int k = 0; k < g.nmem; k++) g.all16 = g.all16 && g.bytes[k] == 16;
  // The position taken from its gathered copy only for double 2D positions.
  if (!(dim == 2 && sizeof(Real) == 8)) g.pos16 = -1;
  if (!with_pos && g.nmem == 0) {
    if (sizeof(Real) == 8 && t.gather_f32_mask) launch_gather_f32(ctx, t, dim, false);
    return;
  }
  float *posf = with_pos ? t.posf : nullptr;
  if (dim == 2) {
    k_gather<Real, 2><<<nb, B, 0, s>>>(t.n, t.order, pos, posf, g);
  } else {
    k_gather<Real, 3><<<nb, B, 0, s>>>(t.n, t.order, pos, posf, g);
  }
  ctx->launches++;
  if (sizeof(Real) == 8 && (t.gather_f32_mask || t.gather_pos_lo))
    launch_gather_f32(ctx, t, dim, with_pos);
}

// Whether a grid may compute cell coordinates in FP32 (k_bin_assign).  The
// grid's cells are wider than its radius by 2^-10, so two agents within the
// radius (as the reference's float-rounded test decides it, at most 2^-22
// beyond) have exact cell coordinates less than 1 - 9.7e-4 apart, and their
// cells differ by at most one whenever each computed coordinate is within
// 4.8e-4 of the exact one.  FP32 rounds x, lo and 1/w (relative u = 2^-24
// each), the difference and the product: for a point inside the grid the
// error is at most (|x| + |lo|) inv u + 3 n u <= (2 |lo| inv + 4 n) u, with
// n the cells along the axis.  Points outside clamp into border cells, which
// keeps them in order.  FP32 is used when that bound is below 2.4e-4, half
// the allowance; queries that compute their cell in FP64 stay consistent.
// Whether a grid (origin lo, 1 / cell size, cells per axis) may compute cell
// coordinates in FP32: the bound on the FP32 rounding error, (2|lo|/w +
// 4n) 2^-24 cell widths, stays within half the cells' 2^-10 margin.
bool fp32_cells_ok(const double *lo, double inv_cell, const int *dims, int dim) {
  for (int d = 0; d < dim; d++) {
    const double bound = (2.0 * std::fabs(lo[d]) * inv_cell + 4.0 * dims[d]) * 5.9604644775390625e-8;
    if (!(bound <= 2.4e-4)) return false;
  }
  return true;
}

bool bin_in_fp32(const TypeState &t, int dim) {
  const int dims[3] = {t.nx, t.ny, t.nz};
  return fp32_cells_ok(t.lo, t.inv_cell, dims, dim);
}

template <typename Real>
void launch_bin(abl_ctx *ctx, TypeState &t, int dim) {
  cudaStream_t s = ctx->stream;
  const int B = 256;
  long nb = blocks_for(t.n, B);
  const Real *pos = (const Real *) t.cols[t.cur][t.d->position_member];
  cudaMemsetAsync(t.cell_count, 0, sizeof(int) * t.ncells, s);
  cudaMemsetAsync(t.amax, 0, sizeof(float), s);
  const bool f32 = bin_in_fp32(t, dim);
#define ABL_BIN_ASSIGN(D, F)                                                                   \
  k_bin_assign<Real, D, F><<<nb, B, 0, s>>>(pos, t.n, t.nx, t.ny, t.nz, t.lo[0], t.lo[1],    \
                                            t.lo[2], t.inv_cell, t.cell_of, t.cell_count,     \
                                            t.local_rank, t.amax, ctx->error)
  if (dim == 2 && f32) ABL_BIN_ASSIGN(2, true);
  else if (dim == 2) ABL_BIN_ASSIGN(2, false);
  else if (f32) ABL_BIN_ASSIGN(3, true);
  else ABL_BIN_ASSIGN(3, false);
#undef ABL_BIN_ASSIGN
  ctx->launches++;
  scan_run(ctx, t.cell_scan, t.cell_count, t.cell_start);
  k_bin_scatter<<<nb, B, 0, s>>>(t.n, t.cell_of, t.local_rank, t.cell_start, t.order);
  ctx->launches++;
  k_cell_sort<<<blocks_for(t.ncells, B), B, 0, s>>>(t.ncells, t.cell_start, t.order);
  ctx->launches++;
  launch_gather<Real>(ctx, t, dim, true);
  if (t.ordered || t.rows) {
    GridGeom geo{t.nx, t.ny, t.nz, t.R};
    build_lists(ctx, geo, dim, t.ordered ? dim : 1, t.R, t.ncells, t.cell_start, t.order,
                t.posf, t.sep, t.nb_cnt, t.nb_scan, t.nb_off, t.nb_list, t.n, t.cell_of);
  }
}

void bin_type(abl_ctx *ctx, TypeState &t) {
  t.bin_id = ++ctx->bin_serial;
  if (pos_is_double(t)) {
    launch_bin<double>(ctx, t, t.d->dim);
  } else {
    launch_bin<float>(ctx, t, t.d->dim);
  }
  t.dirty = false;
  t.regather = false;
}

// Brings a grid up to date with its agent type: a full binning, or only the
// slot-ordered copies of the gathered members when positions did not change.
void bin_grid(abl_ctx *ctx, int gi) {
  TypeState &g = ctx->grids[gi];
  const TypeState &t = ctx->types[ctx->grid_type[gi]];
  for (int b = 0; b < 2; b++)
    for (int k = 0; k < ABL_MAX_MEMBERS; k++) g.cols[b][k] = t.cols[b][k];
  g.cur = t.cur;
  g.n = t.n;
  if (g.dirty) {
    bin_type(ctx, g);
  } else if (g.regather) {
    if (pos_is_double(g)) launch_gather<double>(ctx, g, g.d->dim, false);
    else launch_gather<float>(ctx, g, g.d->dim, false);
    g.regather = false;
  }
}

// The population of type ti changed: every grid of it must be rebuilt.
void mark_dirty(abl_ctx *ctx, int ti) {
  ctx->types[ti].dirty = true;
  for (size_t gi = 0; gi < ctx->grids.size(); gi++) {
    if (ctx->grid_type[gi] == ti) ctx->grids[gi].dirty = true;
  }
}

// Whether no step function ever moves agents of type ti: none may set its
// position member to anything but the agent's own position (`out.pos =
// in.pos` is allowed) and none removes or adds agents of it.  Both buffers
// then hold the uploaded positions for good (CPrinter.cpp:210-213 copies the
// double buffer once; members a step does not write keep their values).
bool positions_static(const abl_model_desc *m, int ti) {
  const abl_agent_desc &a = m->agents[ti];
  if (a.position_member < 0) return false;
  for (int k = 0; k < m->num_steps; k++) {
    const abl_step_desc &sd = m->steps[k];
    if (sd.add_type == ti) return false;
    if (sd.agent_type != ti) continue;
    if (sd.uses_remove || sd.add_type >= 0) return false;
    if (sd.out_changed & (1u << a.position_member)) return false;
  }
  return true;
}

// Members of type ti that keep their uploaded values for good: no step
// function writes them except as `out.m = in.m`, and no step adds or removes
// agents of the type.  Once both buffers hold them (the upload copies them),
// step kernels need not store them.
uint32_t invariant_members(const abl_model_desc *m, int ti) {
  const abl_agent_desc &a = m->agents[ti];
  uint32_t changed = 0;
  for (int k = 0; k < m->num_steps; k++) {
    const abl_step_desc &sd = m->steps[k];
    if (sd.add_type == ti) return 0;
    if (sd.agent_type != ti) continue;
    if (sd.uses_remove || sd.add_type >= 0) return 0;
    changed |= sd.out_changed;
  }
  const uint32_t all = a.num_members >= 32 ? ~0u : (1u << a.num_members) - 1;
  return all & ~changed;
}

// A step function (without population changes) changed members `written`
// of type ti.  Grids of a type whose positions never change keep their
// binning and only re-gather (if they copy a changed member); every other
// grid is rebuilt.
void mark_written(abl_ctx *ctx, int ti, uint32_t written) {
  if (!positions_static(ctx->model, ti)) {
    mark_dirty(ctx, ti);
    return;
  }
  ctx->types[ti].dirty = true;
  for (size_t gi = 0; gi < ctx->grids.size(); gi++) {
    TypeState &g = ctx->grids[gi];
    if (ctx->grid_type[gi] == ti && (g.gather_mask & written)) g.regather = true;
  }
}

void type_amax(abl_ctx *ctx, TypeState &t) {
  cudaStream_t s = ctx->stream;
  const int B = 256;
  cudaMemsetAsync(t.amax, 0, sizeof(float), s);
  long nb = blocks_for(t.n, B);
  const void *pos = t.cols[t.cur][t.d->position_member];
  bool dbl = pos_is_double(t);
  if (t.d->dim == 2) {
    if (dbl) k_amax<double, 2><<<nb, B, 0, s>>>((const double *) pos, t.n, t.amax, ctx->error);
    else k_amax<float, 2><<<nb, B, 0, s>>>((const float *) pos, t.n, t.amax, ctx->error);
  } else {
    if (dbl) k_amax<double, 3><<<nb, B, 0, s>>>((const double *) pos, t.n, t.amax, ctx->error);
    else k_amax<float, 3><<<nb, B, 0, s>>>((const float *) pos, t.n, t.amax, ctx->error);
  }
  ctx->launches++;
}

void drop_graph(abl_ctx *ctx);

__global__ void k_iota(int *a, long n) {
  const long i = (long) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = (int) i;
}

// ------------------------------------------------- kept neighbour lists
//
// When no step function moves agents of a type (and none adds or removes
// them), the set of agents within a constant radius of each agent is the
// same at every timestep.  A near loop around the step's own agent then
// reads its neighbours from a list per agent, found once per binning: the
// candidates are the (2R+1)^DIM cells around the agent's cell, as for the
// step kernels' own search, and the test is the reference's own near test.

__device__ __forceinline__ double nc_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float nc_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double nc_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float nc_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float nc_float(double a) { return __double2float_rn(a); }
__device__ __forceinline__ float nc_float(float a) { return a; }

// Whether agent j is a neighbour of agent i: !(dist(j.pos, i.pos) > radius),
// dist = sqrtf((float) (vx*vx + vy*vy [+ vz*vz])) in the position's type
// (asset/c/libabl.h:156-167; the near test of src/backend/CPrinter.cpp:160-170).  The
// radius is the step's radius expression in that type, widened to double.
template <typename Real, int DIM>
__device__ __forceinline__ bool nc_within(const Real *pos, long i, long j, double radius) {
  Real s = 0;
#pragma unroll
  for (int d = 0; d < DIM; d++) {
    const Real v = pos[DIM * j + d] - pos[DIM * i + d];
    s = d == 0 ? nc_mul(v, v) : nc_add(s, nc_mul(v, v));
  }
  const float f = __fsqrt_rn(nc_float(s));
  return !((double) f > radius);
}

// Pass 1 (list == nullptr): count[i] = agent i's neighbours.  Pass 2: their
// agent indices from list[off[i]], ascending (the order the reference visits
// them in), the largest |neighbour - i| folded into *span, and agent i's
// float position (as the grid's slot-ordered copy rounds it) into posf.
// Candidates are prefiltered as the step kernels do: the FP32 distance of the
// float copies (`slot_posf`, slot order) outside the error band of the radius
// decides; inside it the reference test does.
template <typename Real, int DIM>
__global__ void k_nc_lists(const Real *pos, long n, const int *cell_of, const int *cell_start,
                           const int *order, const float *slot_posf, const float *amax,
                           int nx, int ny, int nz, int R, double radius,
                           int *count, const int *off, int *list, int *span, float *posf) {
  const long i = (long) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const abl::band bd = abl::make_band(radius, *amax, DIM);
  float pf[DIM];
#pragma unroll
  for (int d = 0; d < DIM; d++) pf[d] = (float) pos[DIM * i + d];
  const int l = cell_of[i];
  const int nxy = nx * ny;
  const int c2 = l / nxy, c1 = (l - c2 * nxy) / nx, c0 = l - c2 * nxy - c1 * nx;
  const int z0 = DIM == 3 ? max(c2 - R, 0) : 0, z1 = DIM == 3 ? min(c2 + R, nz - 1) : 0;
  const int y0 = max(c1 - R, 0), y1 = min(c1 + R, ny - 1);
  const int x0 = max(c0 - R, 0), x1 = min(c0 + R, nx - 1);
  int k = 0;
  int *out = list ? list + off[i] : nullptr;
  for (int z = z0; z <= z1; z++) {
    for (int y = y0; y <= y1; y++) {
      const int base = (z * ny + y) * nx;
      const int e = cell_start[base + x1 + 1];
      for (int s = cell_start[base + x0]; s < e; s++) {
        float d2 = 0.0f;
#pragma unroll
        for (int d = 0; d < DIM; d++) {
          const float dd = slot_posf[DIM * s + d] - pf[d];
          d2 = __fadd_rn(d2, __fmul_rn(dd, dd));
        }
        if (d2 > bd.hi) continue;
        const int j = order[s];
        if (!(d2 < bd.lo) && !nc_within<Real, DIM>(pos, i, j, radius)) continue;
        if (out) out[k] = j;
        k++;
      }
    }
  }
  if (!out) {
    count[i] = k;
    return;
  }
  int far = 0;
  for (int a = 0; a < k; a++) {
    const int v = out[a];
    far = max(far, abs(v - (int) i));
    int b = a - 1;
    while (b >= 0 && out[b] > v) {
      out[b + 1] = out[b];
      b--;
    }
    out[b + 1] = v;
  }
  atomicMax(span, far);
#pragma unroll
  for (int d = 0; d < DIM; d++) posf[DIM * i + d] = (float) pos[DIM * i + d];
}

// The int16 form of the lists: entry - owning agent's index.
__global__ void k_nc_narrow(long n, const int *off, const int *list, short *narrow) {
  const long i = (long) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int k = off[i]; k < off[i + 1]; k++) narrow[k] = (short) (list[k] - (int) i);
}

template <typename Real>
void launch_nc_lists(abl_ctx *ctx, const TypeState &g, double radius, int *count, const int *off,
                     int *list, int *span, float *posf) {
  const int B = 128;
  const Real *pos = (const Real *) g.cols[g.cur][g.d->position_member];
  const long nb = blocks_for(g.n, B);
  if (g.d->dim == 2) {
    k_nc_lists<Real, 2><<<nb, B, 0, ctx->stream>>>(pos, g.n, g.cell_of, g.cell_start, g.order,
                                                   g.posf, g.amax, g.nx, g.ny, g.nz, g.R,
                                                   radius, count, off, list, span, posf);
  } else {
    k_nc_lists<Real, 3><<<nb, B, 0, ctx->stream>>>(pos, g.n, g.cell_of, g.cell_start, g.order,
                                                   g.posf, g.amax, g.nx, g.ny, g.nz, g.R,
                                                   radius, count, off, list, span, posf);
  }
  ctx->launches++;
}

// Whether step k keeps its neighbour lists.
bool near_cache_wanted(const abl_ctx *ctx, const abl_step_desc &sd) {
  // Kept lists index neighbours by agent; the float copies of the mixed
  // form are slot-ordered, so such loops search the grid.
  return ctx->near_cache && sd.near_cacheable && sd.agent_type == sd.near_type
      && positions_static(ctx->model, sd.agent_type) && !sd.near_members_f32
      && !sd.near_pos_lo;
}

void nc_release(abl_ctx *ctx, StepState &st, void *p) {
  dev_free(ctx, p);
  st.nc_allocs.erase(std::remove(st.nc_allocs.begin(), st.nc_allocs.end(), p),
                     st.nc_allocs.end());
}

void nc_free_all(abl_ctx *ctx, StepState &st) {
  for (void *p : st.nc_allocs) dev_free(ctx, p);
  st.nc_allocs.clear();
  st.nc_scan.levels.clear();
  st.nc_off = st.nc_count = st.nc_span = st.nc_wide = nullptr;
  st.nc_short = nullptr;
  st.nc_posf = nullptr;
  st.nc_list = nullptr;
  st.nc_n = st.nc_wide_cap = st.nc_short_cap = 0;
}

// Brings step k's kept lists up to date with grid g and returns whether they
// can be read.  Building needs host reads (the total, the index span), so a
// stream capture only reads lists that are already current.  A rebuild
// reuses the buffers it fits in; graphs captured before are dropped when the
// buffers the step kernels read move, or when the lists are given up.
int near_cache_ready(abl_ctx *ctx, int k, const TypeState &g, double radius, bool &ready) {
  ready = false;
  StepState &st = ctx->step_state[k];
  if (!g.dirty && st.nc_bin == g.bin_id && st.nc_radius == radius) {
    ready = st.nc_list != nullptr;
    return ABL_OK;
  }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(ctx->stream, &cs);
  if (cs != cudaStreamCaptureStatusNone || g.dirty) return ABL_OK;
  st.nc_bin = g.bin_id;
  st.nc_radius = radius;
  const void *prev_list = st.nc_list;
  st.nc_list = nullptr;
  auto give_up = [&]() {
    nc_free_all(ctx, st);
    drop_graph(ctx);
    return ABL_OK;  // no room, or lists too long: the step searches the grid
  };
  if (g.n <= 0) return give_up();
  auto *own = &st.nc_allocs;
  bool moved = false;
  if (st.nc_n != g.n) {
    nc_free_all(ctx, st);
    moved = true;
    if (dev_alloc_t(ctx, &st.nc_count, g.n, own) != ABL_OK
        || dev_alloc_t(ctx, &st.nc_off, g.n + 1, own) != ABL_OK
        || dev_alloc_t(ctx, &st.nc_span, 1, own) != ABL_OK
        || dev_alloc_t(ctx, &st.nc_posf, g.n * g.d->dim, own) != ABL_OK
        || scan_plan(ctx, st.nc_scan, g.n, own) != ABL_OK)
      return give_up();
    st.nc_n = g.n;
  }
  const bool dbl = pos_is_double(g);
  if (dbl) launch_nc_lists<double>(ctx, g, radius, st.nc_count, nullptr, nullptr, nullptr, nullptr);
  else launch_nc_lists<float>(ctx, g, radius, st.nc_count, nullptr, nullptr, nullptr, nullptr);
  scan_run(ctx, st.nc_scan, st.nc_count, st.nc_off);
  int total = 0;
  ABL_CUDA_TRY(cudaMemcpyAsync(&total, st.nc_off + g.n, sizeof(int), cudaMemcpyDeviceToHost,
                               ctx->stream));
  ABL_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  // Lists far longer than a handful of cells' worth are not worth keeping.
  if (total < 0 || (long) total > 64 * g.n + 4096) return give_up();
  if (st.nc_wide_cap < std::max(total, 1)) {
    if (st.nc_wide) nc_release(ctx, st, st.nc_wide);
    st.nc_wide = nullptr;
    st.nc_wide_cap = 0;
    if (dev_alloc_t(ctx, &st.nc_wide, std::max(total, 1), own) != ABL_OK) return give_up();
    st.nc_wide_cap = std::max(total, 1);
  }
  ABL_CUDA_TRY(cudaMemsetAsync(st.nc_span, 0, sizeof(int), ctx->stream));
  if (dbl) launch_nc_lists<double>(ctx, g, radius, nullptr, st.nc_off, st.nc_wide, st.nc_span,
                                   st.nc_posf);
  else launch_nc_lists<float>(ctx, g, radius, nullptr, st.nc_off, st.nc_wide, st.nc_span,
                              st.nc_posf);
  int far = 0;
  ABL_CUDA_TRY(cudaMemcpyAsync(&far, st.nc_span, sizeof(int), cudaMemcpyDeviceToHost,
                               ctx->stream));
  ABL_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  st.nc_list = st.nc_wide;
  st.nc_narrow = false;
  if (far <= 32767) {
    if (st.nc_short_cap < std::max(total, 1)) {
      if (st.nc_short) nc_release(ctx, st, st.nc_short);
      st.nc_short = nullptr;
      st.nc_short_cap = 0;
      if (dev_alloc_t(ctx, &st.nc_short, std::max(total, 1), own) == ABL_OK)
        st.nc_short_cap = std::max(total, 1);
    }
    if (st.nc_short) {
      k_nc_narrow<<<blocks_for(g.n, 256), 256, 0, ctx->stream>>>(g.n, st.nc_off, st.nc_wide,
                                                                   st.nc_short);
      ctx->launches++;
      st.nc_list = st.nc_short;
      st.nc_narrow = true;
    }
  }
  if (moved || st.nc_list != prev_list) drop_graph(ctx);
  ready = true;
  return ABL_OK;
}

// One iteration of the simulate loop (src/backend/CPrinter.cpp:189-233).
int step_once(abl_ctx *ctx) {
  const abl_model_desc *m = ctx->model;
  if (m->seq_step) cudaEventRecord(ctx->ts0, ctx->stream);
  for (int k = 0; k < m->num_steps; k++) {
    const abl_step_desc &sd = m->steps[k];
    TypeState &t = ctx->types[sd.agent_type];
    abl_step_launch L;
    std::memset(&L, 0, sizeof L);
    L.n = t.n;
    L.globals = ctx->globals.data();
    L.error = ctx->error;
    L.block = 128;
    L.seed = ctx->seed;
    L.timestep = ctx->timestep;
    L.step_index = k;
    L.skip_store = ctx->skip_stores ? invariant_members(m, sd.agent_type) : 0;
    // Steps that draw random numbers in sequential mode: one agent per
    // launch, in index order.
    const bool serial = ctx->serial_rng && sd.uses_rng && t.n > 0;
    if (serial) {
      L.serial_rng = ctx->serial_rng;
      if (ctx->serial_iota_n < t.n) {
        if (ctx->serial_iota) dev_free(ctx, ctx->serial_iota);
        ctx->serial_iota = nullptr;
        ctx->serial_iota_n = 0;
        ABL_TRY(dev_alloc_t(ctx, &ctx->serial_iota, t.n));
        k_iota<<<blocks_for(t.n, 256), 256, 0, ctx->stream>>>(ctx->serial_iota, t.n);
        ctx->launches++;
        ctx->serial_iota_n = t.n;
      }
    }
    bool changes = sd.uses_remove || sd.add_type >= 0;
    if (changes) {
      StepState &st = ctx->step_state[k];
      L.removed = st.removed;
      L.child_flag = st.child_flag;
      for (int j = 0; j < ABL_MAX_MEMBERS; j++) L.child_cols[j] = st.child_cols[j];
    }
    for (int j = 0; j < t.d->num_members; j++) {
      L.in_cols[j] = t.cols[t.cur][j];
      L.out_cols[j] = t.cols[1 - t.cur][j];
    }
    if (sd.near_type >= 0) {
      int gi = ctx->step_grid[k];
      TypeState &nt = ctx->grids[gi];
      // Kept lists read the step's own columns: a grid that only needs its
      // slot-ordered copies refreshed is left as it is.
      bool cached = false;
      if (nt.dirty) {
        Phase ph("bin");
        bin_grid(ctx, gi);
      }
      if (near_cache_wanted(ctx, sd)) {
        Phase ph("kept lists");
        ABL_TRY(near_cache_ready(ctx, k, nt, sd.radius(ctx->globals.data()), cached));
      }
      if (!cached && nt.regather) {
        Phase ph("gather");
        bin_grid(ctx, gi);
      }
      abl_near_view &V = L.near;
      const int depth = list_depth(sd, *nt.d, ctx->near_mode);
      V.dim = nt.d->dim;
      V.ordered = depth == 2;
      V.rows = depth == 1 ? nt.sep.elem[0] : nullptr;
      V.row_off = nt.sep.off[0];
      V.range = nt.R;
      V.nx = nt.nx;
      V.ny = nt.ny;
      V.nz = nt.nz;
      for (int d = 0; d < 3; d++) V.lo[d] = nt.lo[d];
      V.inv_cell = nt.inv_cell;
      V.radius = sd.radius(ctx->globals.data());
      V.n = nt.n;
      V.cell_start = nt.cell_start;
      V.order = nt.order;
      V.posf = nt.posf;
      V.nb_off = nt.nb_off;
      V.nb_list = nt.nb_list;
      for (int j = 0; j < nt.d->num_members; j++) {
        V.cols[j] = nt.gcols[j];
        V.fcols[j] = nt.fcols[j];
      }
      V.poslo = nt.poslo;
      V.balance = ctx->balance;
      V.cap = V.ordered ? ctx->list_cap : ctx->runs_cap;
      V.cell_of = sd.agent_type == sd.near_type ? nt.cell_of : nullptr;
      V.cell_base = 0;
      V.cell_f32 = bin_in_fp32(nt, nt.d->dim) ? 1 : 0;
      // Threads visit the binned agents in slot order, so a block's agents
      // fill consecutive cells: block lists pay off.
      V.block_cap = block_lists_wanted(sd, depth, ctx->near_mode) ? ctx->block_cap : 0;
      if (cached) {
        // Kept lists: agents in index order, neighbours read by index from
        // the step's own columns, no block lists.
        const StepState &st = ctx->step_state[k];
        V.ncache_off = st.nc_off;
        V.ncache_list = st.nc_list;
        V.ncache_narrow = st.nc_narrow ? 1 : 0;
        V.posf = st.nc_posf;
        for (int j = 0; j < t.d->num_members; j++) V.cols[j] = t.cols[t.cur][j];
        V.block_cap = 0;
      }
      if (sd.presorted) L.smem = abl::presort_bytes(V);
      if (sd.agent_type == sd.near_type) {
        V.amax = nt.amax;
        L.visit_order = cached ? nullptr : nt.order;
      } else {
        if (t.d->position_member >= 0 && t.n > 0) {
          type_amax(ctx, t);
          k_max2<<<1, 1, 0, ctx->stream>>>(t.amax, nt.amax, ctx->amax_pair);
          ctx->launches++;
          V.amax = ctx->amax_pair;
        } else {
          V.amax = nt.amax;
        }
      }
    }
    if (t.n > 0) {
      Phase ph(sd.name);
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      cudaStreamIsCapturing(ctx->stream, &cs);
      bool timed = ctx->profile && cs == cudaStreamCaptureStatusNone;
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      if (timed) {
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, ctx->stream);
      }
      if (serial) {
        abl_step_launch L1 = L;
        L1.n = 1;
        L1.block = 1;
        L1.near.block_cap = 0;
        L1.near.balance = 0;
        if (sd.presorted && sd.near_type >= 0) L1.smem = abl::presort_bytes(L1.near);
        for (long i = 0; i < t.n; i++) {
          L1.visit_order = ctx->serial_iota + i;
          ABL_TRY(sd.launch(&L1, ctx->stream));
          ctx->launches++;
        }
      } else {
        ABL_TRY(sd.launch(&L, ctx->stream));
        ctx->launches++;
      }
      if (timed) {
        cudaEventRecord(e1, ctx->stream);
        ctx->prof_pending[k].push_back({e0, e1});
      }
    }
    if (changes) {
      Phase ph("compact");
      bool regrow = false;
      ABL_TRY(apply_population_changes(ctx, k, regrow));
      if (regrow) ABL_TRY(prepare(ctx));
    } else {
      t.cur = 1 - t.cur;  // swap agents_X and agents_X_dbuf
      mark_written(ctx, sd.agent_type, sd.out_changed);
    }
  }
  ctx->timestep++;
  if (m->seq_step) {
    // The sequential step runs on the host after the parallel steps
    // (src/AnalysisVisitor.cpp:695-704), with this timestep's device time.
    cudaEventRecord(ctx->ts1, ctx->stream);
    ABL_CUDA_TRY(cudaEventSynchronize(ctx->ts1));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ctx->ts0, ctx->ts1);
    ctx->last_timestep = ms / 1000.0;
    ctx->seq_error = 0;
    ABL_TRY(m->seq_step(ctx, ctx->globals.data()));
    if (ctx->seq_error) return ctx->seq_error;
  }
  return ABL_OK;
}

bool graph_capturable(const abl_ctx *ctx) {
  const abl_model_desc *m = ctx->model;
  if (m->seq_step) return false;
  for (int k = 0; k < m->num_steps; k++) {
    // Population changes need host decisions; random() keys on the timestep,
    // which a replayed graph would not advance.
    if (m->steps[k].uses_remove || m->steps[k].add_type >= 0 || m->steps[k].uses_rng)
      return false;
  }
  return true;
}

int check_error(abl_ctx *ctx) {
  if (ctx->error_host) {
    // One round trip: the error word follows the stream's work into pinned
    // memory, then a single synchronisation.
    ABL_CUDA_TRY(cudaMemcpyAsync(ctx->error_host, ctx->error, sizeof(int),
                                 cudaMemcpyDeviceToHost, ctx->stream));
    ABL_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    const int e = *ctx->error_host;
    if (e != 0) {
      cudaMemsetAsync(ctx->error, 0, sizeof(int), ctx->stream);
      cudaStreamSynchronize(ctx->stream);
      return e;
    }
    return ABL_OK;
  }
  ABL_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  int h = 0;
  ABL_CUDA_TRY(cudaMemcpy(&h, ctx->error, sizeof(int), cudaMemcpyDeviceToHost));
  if (h != 0) {
    int zero = 0;
    cudaMemcpy(ctx->error, &zero, sizeof(int), cudaMemcpyHostToDevice);
    return h;
  }
  return ABL_OK;
}

void drop_graph(abl_ctx *ctx) {
  for (auto &g : ctx->graphs) cudaGraphExecDestroy(g.exec);
  ctx->graphs.clear();
  ctx->warm = false;
}

std::vector<int> graph_key(const abl_ctx *ctx) {
  std::vector<int> key;
  for (const TypeState &t : ctx->types) {
    key.push_back(t.cur);
    key.push_back(t.dirty ? 1 : 0);
  }
  for (const TypeState &g : ctx->grids) key.push_back((g.dirty ? 1 : 0) | (g.regather ? 2 : 0));
  return key;
}

// Collects finished per-kernel timings.
void collect_profile(abl_ctx *ctx) {
  for (size_t k = 0; k < ctx->prof_pending.size(); k++) {
    for (auto &ev : ctx->prof_pending[k]) {
      float ms = 0.0f;
      if (cudaEventElapsedTime(&ms, ev.first, ev.second) == cudaSuccess) {
        ctx->prof_seconds[k] += ms / 1000.0;
        ctx->prof_launches[k]++;
      }
      cudaEventDestroy(ev.first);
      cudaEventDestroy(ev.second);
    }
    ctx->prof_pending[k].clear();
  }
}

void apply_key(abl_ctx *ctx, const std::vector<int> &key) {
  for (size_t k = 0; k < ctx->types.size(); k++) {
    ctx->types[k].cur = key[2 * k];
    ctx->types[k].dirty = key[2 * k + 1] != 0;
  }
  for (size_t q = 0; q < ctx->grids.size(); q++) {
    ctx->grids[q].dirty = (key[2 * ctx->types.size() + q] & 1) != 0;
    ctx->grids[q].regather = (key[2 * ctx->types.size() + q] & 2) != 0;
  }
}

// Captures `steps` timesteps into a CUDA graph, or returns the one captured
// from this state.  The graph's buffers are those of the state it starts
// from; after replaying it the context is in the graph's end state (the same
// state again for two timesteps, where every double buffer swaps twice).
abl_ctx::Graph *find_graph(abl_ctx *ctx, int steps) {
  std::vector<int> key = graph_key(ctx);
  key.push_back(steps);
  for (auto &g : ctx->graphs) {
    if (g.key == key) return &g;
  }
  return nullptr;
}

int capture_graph(abl_ctx *ctx, int steps, abl_ctx::Graph **out) {
  if ((*out = find_graph(ctx, steps)) != nullptr) return ABL_OK;
  std::vector<int> key = graph_key(ctx);
  key.push_back(steps);
  abl_ctx::Graph G;
  G.key = key;
  G.steps = steps;
  cudaGraph_t g = nullptr;
  long before = ctx->launches;
  const long timestep = ctx->timestep;
  ABL_CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  int r = ABL_OK;
  for (int k = 0; k < steps && r == ABL_OK; k++) r = step_once(ctx);
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  G.end_key = graph_key(ctx);
  ctx->timestep = timestep;
  if (r != ABL_OK) {
    if (g) cudaGraphDestroy(g);
    return r;
  }
  ABL_CUDA_TRY(e);
  e = cudaGraphInstantiate(&G.exec, g, 0);
  cudaGraphDestroy(g);
  ABL_CUDA_TRY(e);
  G.launches = ctx->launches - before;
  ctx->launches = before;
  // Capturing does not run anything: restore the state the graph starts from.
  apply_key(ctx, key);
  ctx->graphs.push_back(G);
  *out = &ctx->graphs.back();
  return ABL_OK;
}

}  // namespace

extern "C" {

extern const abl_model_desc *const abl_builtin_models[];

const abl_model_desc *abl_model_lookup(const char *name) {
  if (!name) return nullptr;
  for (int k = 0; abl_builtin_models[k]; k++) {
    if (std::strcmp(abl_builtin_models[k]->name, name) == 0) return abl_builtin_models[k];
  }
  return nullptr;
}

int abl_model_num_agent_types(const abl_model_desc *m) { return m ? m->num_agent_types : ABL_E_INVALID; }

const char *abl_model_agent_name(const abl_model_desc *m, int type_id) {
  if (!m || type_id < 0 || type_id >= m->num_agent_types) return nullptr;
  return m->agents[type_id].name;
}

int abl_model_num_members(const abl_model_desc *m, int type_id) {
  if (!m || type_id < 0 || type_id >= m->num_agent_types) return ABL_E_INVALID;
  return m->agents[type_id].num_members;
}

int abl_model_member(const abl_model_desc *m, int type_id, int member, const char **name,
                     int *value_type) {
  if (!m || type_id < 0 || type_id >= m->num_agent_types) return ABL_E_INVALID;
  const abl_agent_desc &a = m->agents[type_id];
  if (member < 0 || member >= a.num_members) return ABL_E_INVALID;
  if (name) *name = a.members[member].name;
  if (value_type) *value_type = a.members[member].value_type;
  return ABL_OK;
}

size_t abl_model_globals_size(const abl_model_desc *m) { return m ? m->globals_size : 0; }

int abl_model_float_bytes(const abl_model_desc *m) {
  if (!m) return ABL_E_INVALID;
  return m->uses_float ? 4 : 8;
}

int abl_model_globals_default(const abl_model_desc *m, void *out) {
  if (!m || !out) return ABL_E_INVALID;
  std::memcpy(out, m->globals_default, m->globals_size);
  return ABL_OK;
}

int abl_model_global(const abl_model_desc *m, const char *name, size_t *offset, int *value_type) {
  if (!m || !name) return ABL_E_INVALID;
  for (int k = 0; k < m->num_globals; k++) {
    if (std::strcmp(m->globals[k].name, name) == 0) {
      if (offset) *offset = m->globals[k].offset;
      if (value_type) *value_type = m->globals[k].value_type;
      return ABL_OK;
    }
  }
  return ABL_E_INVALID;
}

int abl_create(const abl_model_desc *model, size_t hbm_budget, abl_ctx **out) {
  if (!model || !out) return ABL_E_INVALID;
  if (model->num_agent_types <= 0) return ABL_E_INVALID;
  abl_ctx *ctx = new abl_ctx;
  ctx->model = model;
  ctx->budget = hbm_budget;
  ctx->globals.assign((const unsigned char *) model->globals_default,
                      (const unsigned char *) model->globals_default + model->globals_size);
  ctx->types.resize(model->num_agent_types);
  for (int k = 0; k < model->num_steps; k++) {
    const abl_step_desc &sd = model->steps[k];
    if (sd.uses_remove) ctx->types[sd.agent_type].dynamic = true;
    if (sd.add_type >= 0) ctx->types[sd.add_type].dynamic = true;
  }
  for (int k = 0; k < model->num_agent_types; k++) {
    ctx->types[k].d = &model->agents[k];
    if (model->agents[k].num_members > ABL_MAX_MEMBERS) {
      delete ctx;
      return ABL_E_UNSUPPORTED;
    }
  }
  cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ts0);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ts1);
  if (e == cudaSuccess) e = take_error_slot(&ctx->error_host);
  if (e != cudaSuccess) {
    std::fprintf(stderr, "openabl-cuda: context setup failed: %s\n", cudaGetErrorString(e));
    delete ctx;
    return ABL_E_CUDA;
  }
  int r = dev_alloc_t(ctx, &ctx->error, 1);
  if (r == ABL_OK) r = cudaMemsetAsync(ctx->error, 0, sizeof(int), ctx->stream) == cudaSuccess
                           ? ABL_OK : ABL_E_CUDA;
  if (r != ABL_OK) {
    abl_destroy(ctx);
    return r;
  }
  *out = ctx;
  return ABL_OK;
}

int abl_set_globals(abl_ctx *ctx, const void *globals, size_t size) {
  if (!ctx || !globals || size != ctx->model->globals_size) return ABL_E_INVALID;
  std::memcpy(ctx->globals.data(), globals, size);
  ctx->prepared = false;
  drop_graph(ctx);
  return ABL_OK;
}

// Sizes both buffers of a type for n agents (types whose population changes
// at run time keep spare capacity and reallocate only to grow).
static int size_type(abl_ctx *ctx, TypeState &t, size_t n, bool &resized) {
  long want_cap = t.dynamic ? std::max<long>(2 * (long) n, 1024) : (long) n;
  resized = !t.uploaded || (t.dynamic ? (long) n > t.cap : (long) n != t.n);
  if (resized) {
    for (int b = 0; b < 2; b++) {
      for (int k = 0; k < t.d->num_members; k++) {
        if (t.cols[b][k]) dev_free(ctx, t.cols[b][k]);
        t.cols[b][k] = nullptr;
        ABL_TRY(dev_alloc(ctx, &t.cols[b][k],
                          member_bytes(t.d->members[k]) * std::max<long>(want_cap, 1)));
      }
    }
    t.cap = want_cap;
  }
  t.n = (long) n;
  t.cur = 0;
  return ABL_OK;
}

// Whether the double buffer's copy of member k of type ti can ever be
// read: not when every step function of the type always writes the member
// (its `out` column is overwritten before the buffers swap), nor when no
// step function runs on the type (the buffers never swap).
static bool dbuf_read(const abl_model_desc *m, int ti, int k) {
  if (invariant_members(m, ti) & (1u << k)) return true;  // kernels skip their stores
  for (int s = 0; s < m->num_steps; s++) {
    const abl_step_desc &sd = m->steps[s];
    if (sd.agent_type != ti) continue;
    if (!(sd.out_written & (1u << k))) return true;
  }
  return false;
}

// The state in buffer 0 is the population: the double buffer starts as a
// copy (CPrinter.cpp:210-213) where it can be read, every binning of the
// type is stale.
static int finish_upload(abl_ctx *ctx, int type_id, bool resized) {
  TypeState &t = ctx->types[type_id];
  for (int k = 0; k < t.d->num_members; k++) {
    size_t bytes = member_bytes(t.d->members[k]) * (size_t) t.n;
    if (bytes == 0 || !dbuf_read(ctx->model, type_id, k)) continue;
    ABL_CUDA_TRY(cudaMemcpyAsync(t.cols[1][k], t.cols[0][k], bytes, cudaMemcpyDeviceToDevice,
                                 ctx->stream));
  }
  t.uploaded = true;
  mark_dirty(ctx, type_id);
  // Kept neighbour lists of this type are rebuilt (in place) by an eager
  // timestep before graphs that read them replay again.
  for (int k = 0; k < ctx->model->num_steps && !resized; k++) {
    if (ctx->model->steps[k].near_type == type_id && k < (int) ctx->step_state.size()
        && ctx->step_state[k].nc_list)
      ctx->warm = false;
  }
  if (resized) {
    ctx->prepared = false;
    drop_graph(ctx);
  }
  return ABL_OK;
}

int abl_upload(abl_ctx *ctx, int type_id, const void *const *cols, size_t n) {
  if (!ctx || type_id < 0 || type_id >= (int) ctx->types.size()) return ABL_E_INVALID;
  Phase ph("upload");
  if (n > (size_t) INT32_MAX) return ABL_E_UNSUPPORTED;
  TypeState &t = ctx->types[type_id];
  if (n > 0 && !cols) return ABL_E_INVALID;
  if (n > 0) {
    for (int k = 0; k < t.d->num_members; k++)
      if (member_bytes(t.d->members[k]) > 0 && !cols[k]) return ABL_E_INVALID;
  }
  bool resized = false;
  ABL_TRY(size_type(ctx, t, n, resized));
  for (int k = 0; k < t.d->num_members; k++) {
    size_t bytes = member_bytes(t.d->members[k]) * n;
    if (bytes == 0) continue;
    ABL_CUDA_TRY(cudaMemcpyAsync(t.cols[0][k], cols[k], bytes, cudaMemcpyHostToDevice, ctx->stream));
  }
  return finish_upload(ctx, type_id, resized);
}

int abl_reserve(abl_ctx *ctx, int type_id, size_t n, void **dev_cols) {
  if (!ctx || !dev_cols || type_id < 0 || type_id >= (int) ctx->types.size())
    return ABL_E_INVALID;
  if (n > (size_t) INT32_MAX) return ABL_E_UNSUPPORTED;
  TypeState &t = ctx->types[type_id];
  bool resized = false;
  ABL_TRY(size_type(ctx, t, n, resized));
  t.reserved_resize = t.reserved_resize || resized;
  ABL_CUDA_TRY(cudaStreamSynchronize(ctx->stream));  // buffers free for the caller's writes
  for (int k = 0; k < t.d->num_members; k++) dev_cols[k] = t.cols[0][k];
  return ABL_OK;
}

int abl_commit(abl_ctx *ctx, int type_id) {
  if (!ctx || type_id < 0 || type_id >= (int) ctx->types.size()) return ABL_E_INVALID;
  TypeState &t = ctx->types[type_id];
  if (t.n > 0 && !t.cols[0][0] && t.d->num_members > 0) return ABL_E_INVALID;
  const bool resized = t.reserved_resize || !t.uploaded;
  t.reserved_resize = false;
  return finish_upload(ctx, type_id, resized);
}

static int ensure_ready(abl_ctx *ctx) {
  for (auto &t : ctx->types) {
    if (!t.uploaded) {
      // Types never uploaded have no agents.
      long cap = t.dynamic ? 1024 : 1;
      for (int b = 0; b < 2; b++)
        for (int k = 0; k < t.d->num_members; k++)
          if (!t.cols[b][k])
            ABL_TRY(dev_alloc(ctx, &t.cols[b][k], member_bytes(t.d->members[k]) * cap));
      t.n = 0;
      t.cap = cap;
      t.uploaded = true;
    }
  }
  if (!ctx->prepared) ABL_TRY(prepare(ctx));
  return ABL_OK;
}

int abl_run(abl_ctx *ctx, int timesteps) {
  if (!ctx || timesteps < 0) return ABL_E_INVALID;
  ABL_TRY(ensure_ready(ctx));
  long launches0 = ctx->launches;
  ABL_CUDA_TRY(cudaEventRecord(ctx->ev0, ctx->stream));
  int done = 0;
  const bool graphs = !ctx->profile && graph_capturable(ctx);
  // After an upload or a change of settings the first timestep runs eagerly
  // (it settles which binnings are current); then timesteps replay captured
  // graphs: two at a time, and a one-timestep graph for an odd remainder
  // (so that abl_step replays too).
  if (timesteps > 0 && !(graphs && ctx->warm)) {
    ABL_TRY(step_once(ctx));
    done = 1;
    ctx->warm = true;
  }
  if (graphs) {
    while (timesteps - done > 0) {
      const int steps = timesteps - done >= 2 ? 2 : 1;
      abl_ctx::Graph *G = find_graph(ctx, steps);
      if (!G) {
        // A single timestep is not worth a capture inside the timed region;
        // its graph is captured after it (below).
        if (steps == 1) break;
        ABL_TRY(capture_graph(ctx, steps, &G));
      }
      ABL_CUDA_TRY(cudaGraphLaunch(G->exec, ctx->stream));
      ctx->launches += G->launches;
      apply_key(ctx, G->end_key);
      ctx->timestep += steps;
      done += steps;
    }
  }
  for (; done < timesteps; done++) ABL_TRY(step_once(ctx));
  ABL_CUDA_TRY(cudaEventRecord(ctx->ev1, ctx->stream));
  int r = check_error(ctx);
  if (r == ABL_OK && graphs && ctx->warm && !find_graph(ctx, 1)) {
    abl_ctx::Graph *G = nullptr;
    r = capture_graph(ctx, 1, &G);
  }
  collect_profile(ctx);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  ctx->last_exec = ms / 1000.0;
  ctx->last_launches = ctx->launches - launches0;
  return r;
}

int abl_step(abl_ctx *ctx) { return abl_run(ctx, 1); }

int abl_count(abl_ctx *ctx, int type_id, size_t *n) {
  if (!ctx || !n || type_id < 0 || type_id >= (int) ctx->types.size()) return ABL_E_INVALID;
  *n = (size_t) ctx->types[type_id].n;
  return ABL_OK;
}

int abl_download(abl_ctx *ctx, int type_id, void *const *cols, size_t *n) {
  if (!ctx || !n || type_id < 0 || type_id >= (int) ctx->types.size()) return ABL_E_INVALID;
  Phase ph("download");
  TypeState &t = ctx->types[type_id];
  size_t cnt = (size_t) t.n;
  if (*n < cnt) {
    *n = cnt;
    return ABL_E_INVALID;
  }
  for (int k = 0; k < t.d->num_members; k++) {
    size_t bytes = member_bytes(t.d->members[k]) * cnt;
    if (bytes == 0) continue;
    if (!cols || !cols[k]) return ABL_E_INVALID;
    ABL_CUDA_TRY(cudaMemcpyAsync(cols[k], t.cols[t.cur][k], bytes, cudaMemcpyDeviceToHost,
                                 ctx->stream));
  }
  *n = cnt;
  return check_error(ctx);
}

// ------------------------------------------------- checkpoint and resume
//
// File layout (host byte order): "ABLSTAT1", the model's name (64 bytes),
// the number of agent types, timestep, seed, whether the sequential random
// stream is on and its state, the globals block; then per type its agent
// count and, per member, its bytes per agent followed by the current
// buffer's and the double buffer's first n agents.

namespace {

const char kStateMagic[8] = {'A', 'B', 'L', 'S', 'T', 'A', 'T', '1'};

struct StateHeader {
  char magic[8];
  char model[64];
  int32_t types;
  int32_t serial_on;
  int64_t timestep;
  uint64_t seed;
  uint64_t serial_state[2];
  uint64_t globals_size;
};

struct FileCloser {
  FILE *f;
  ~FileCloser() {
    if (f) std::fclose(f);
  }
};

}  // namespace

int abl_save_state(abl_ctx *ctx, const char *path) {
  if (!ctx || !path) return ABL_E_INVALID;
  ABL_TRY(ensure_ready(ctx));
  StateHeader h;
  std::memset(&h, 0, sizeof h);
  std::memcpy(h.magic, kStateMagic, 8);
  std::snprintf(h.model, sizeof h.model, "%s", ctx->model->name);
  h.types = (int32_t) ctx->types.size();
  h.timestep = ctx->timestep;
  h.seed = ctx->seed;
  h.serial_on = ctx->serial_rng ? 1 : 0;
  if (ctx->serial_rng) ABL_TRY(abl_get_serial_random(ctx, h.serial_state));
  h.globals_size = ctx->globals.size();
  ABL_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  FileCloser fc{std::fopen(path, "wb")};
  if (!fc.f) return ABL_E_IO;
  bool ok = std::fwrite(&h, sizeof h, 1, fc.f) == 1
         && std::fwrite(ctx->globals.data(), 1, ctx->globals.size(), fc.f) == ctx->globals.size();
  std::vector<unsigned char> buf;
  for (const TypeState &t : ctx->types) {
    const int64_t n = t.n;
    const int32_t members = t.d->num_members;
    ok = ok && std::fwrite(&n, sizeof n, 1, fc.f) == 1
            && std::fwrite(&members, sizeof members, 1, fc.f) == 1;
    for (int k = 0; k < t.d->num_members && ok; k++) {
      const uint64_t b = member_bytes(t.d->members[k]);
      ok = std::fwrite(&b, sizeof b, 1, fc.f) == 1;
      const size_t bytes = b * (size_t) n;
      buf.resize(std::max<size_t>(bytes, 1));
      for (int which = 0; which < 2 && ok && bytes > 0; which++) {
        const void *src = t.cols[which == 0 ? t.cur : 1 - t.cur][k];
        ABL_CUDA_TRY(cudaMemcpy(buf.data(), src, bytes, cudaMemcpyDeviceToHost));
        ok = std::fwrite(buf.data(), 1, bytes, fc.f) == bytes;
      }
    }
  }
  ok = ok && std::fflush(fc.f) == 0;
  return ok ? check_error(ctx) : ABL_E_IO;
}

int abl_load_state(abl_ctx *ctx, const char *path) {
  if (!ctx || !path) return ABL_E_INVALID;
  FileCloser fc{std::fopen(path, "rb")};
  if (!fc.f) return ABL_E_IO;
  StateHeader h;
  if (std::fread(&h, sizeof h, 1, fc.f) != 1 || std::memcmp(h.magic, kStateMagic, 8) != 0)
    return ABL_E_IO;
  h.model[sizeof h.model - 1] = 0;
  if (std::strcmp(h.model, ctx->model->name) != 0 || h.types != (int32_t) ctx->types.size()
      || h.globals_size != ctx->globals.size())
    return ABL_E_IO;
  // The whole file is read and checked into host buffers first; the context
  // is changed only once every check has passed, so a truncated or
  // mismatched file leaves it as it was.
  std::vector<unsigned char> globals(h.globals_size);
  if (std::fread(globals.data(), 1, globals.size(), fc.f) != globals.size()) return ABL_E_IO;
  struct TypeImage {
    int64_t n = 0;
    std::vector<std::vector<unsigned char>> cur, dbuf;
  };
  std::vector<TypeImage> img(ctx->types.size());
  for (int ti = 0; ti < (int) ctx->types.size(); ti++) {
    const abl_agent_desc &d = ctx->model->agents[ti];
    int64_t n = 0;
    int32_t members = 0;
    if (std::fread(&n, sizeof n, 1, fc.f) != 1 || std::fread(&members, sizeof members, 1, fc.f) != 1
        || members != d.num_members || n < 0 || n > INT32_MAX)
      return ABL_E_IO;
    TypeImage &T = img[ti];
    T.n = n;
    T.cur.resize(members);
    T.dbuf.resize(members);
    for (int k = 0; k < members; k++) {
      uint64_t b = 0;
      if (std::fread(&b, sizeof b, 1, fc.f) != 1 || b != member_bytes(d.members[k]))
        return ABL_E_IO;
      const size_t bytes = b * (size_t) n;
      T.cur[k].resize(std::max<size_t>(bytes, 1));
      T.dbuf[k].resize(std::max<size_t>(bytes, 1));
      if (bytes > 0 && (std::fread(T.cur[k].data(), 1, bytes, fc.f) != bytes
                        || std::fread(T.dbuf[k].data(), 1, bytes, fc.f) != bytes))
        return ABL_E_IO;
    }
  }
  if (std::fgetc(fc.f) != EOF) return ABL_E_IO;  // trailing bytes: not this model's file
  ABL_TRY(abl_set_globals(ctx, globals.data(), globals.size()));
  for (int ti = 0; ti < (int) ctx->types.size(); ti++) {
    const abl_agent_desc &d = ctx->model->agents[ti];
    TypeImage &T = img[ti];
    std::vector<const void *> cols(d.num_members);
    for (int k = 0; k < d.num_members; k++) cols[k] = T.cur[k].data();
    ABL_TRY(abl_upload(ctx, ti, cols.data(), (size_t) T.n));
    TypeState &t = ctx->types[ti];
    for (int k = 0; k < d.num_members; k++) {
      const size_t bytes = member_bytes(d.members[k]) * (size_t) T.n;
      if (bytes == 0) continue;
      ABL_CUDA_TRY(cudaMemcpyAsync(t.cols[1 - t.cur][k], T.dbuf[k].data(), bytes,
                                   cudaMemcpyHostToDevice, ctx->stream));
    }
    ABL_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  }
  ctx->timestep = h.timestep;
  ctx->seed = h.seed;
  ABL_TRY(abl_set_serial_random(ctx, h.serial_on ? h.serial_state : nullptr));
  drop_graph(ctx);
  return ABL_OK;
}

int abl_reduce(abl_ctx *ctx, int kind, int type_id, int member, void *out) {
  if (!ctx || !out || type_id < 0 || type_id >= (int) ctx->types.size()) return ABL_E_INVALID;
  Phase ph("reduce");
  TypeState &t = ctx->types[type_id];
  if (kind == ABL_REDUCE_COUNT) {
    *(int *) out = (int) t.n;
    return ABL_OK;
  }
  if (member < 0 || member >= t.d->num_members) return ABL_E_INVALID;
  const abl_member_desc &md = t.d->members[member];
  const void *col = t.cols[t.cur][member];
  cudaStream_t s = ctx->stream;
  if (!ctx->d_pair) ABL_TRY(dev_alloc_t(ctx, &ctx->d_pair, 2));
  if (!ctx->d_red) ABL_TRY(dev_alloc_t(ctx, &ctx->d_red, 4));
  if (kind == ABL_REDUCE_SUM) {
    if (md.value_type == ABL_T_BOOL || md.value_type == ABL_T_INT) {
      ABL_CUDA_TRY(cudaMemsetAsync(ctx->d_red, 0, sizeof(double) * 4, s));
      k_sum_int<<<blocks_for(t.n, 256), 256, 0, s>>>(col, md.scalar_bytes, t.n,
                                                     (unsigned long long *) ctx->d_red);
      long long v = 0;
      ABL_CUDA_TRY(cudaMemcpyAsync(&v, ctx->d_red, sizeof v, cudaMemcpyDeviceToHost, s));
      ABL_CUDA_TRY(cudaStreamSynchronize(s));
      *(int *) out = (int) v;
      return ABL_OK;
    }
    // Floating-point members: added in ascending agent order, one thread,
    // so that the result does not depend on the launch configuration.
    k_sum_seq<<<1, 1, 0, s>>>(col, md.scalar_bytes, md.components, t.n, ctx->d_red);
    double v[3] = {0, 0, 0};
    ABL_CUDA_TRY(cudaMemcpyAsync(v, ctx->d_red, sizeof v, cudaMemcpyDeviceToHost, s));
    ABL_CUDA_TRY(cudaStreamSynchronize(s));
    for (int c = 0; c < md.components; c++) {
      if (md.scalar_bytes == 4) ((float *) out)[c] = (float) v[c];
      else ((double *) out)[c] = v[c];
    }
    return ABL_OK;
  }
  if (kind == ABL_REDUCE_COUNT_EQ) {
    unsigned char value[24];
    size_t vb = member_bytes(md);
    std::memcpy(value, out, vb);
    EqArgs a;
    std::memcpy(a.value, value, vb);
    a.bytes = (int) vb;
    a.scalar = md.scalar_bytes;
    a.is_float = md.value_type == ABL_T_FLOAT || md.value_type == ABL_T_FLOAT2
                 || md.value_type == ABL_T_FLOAT3;
    ABL_CUDA_TRY(cudaMemsetAsync(ctx->d_red, 0, sizeof(double) * 4, s));
    k_count_eq<<<blocks_for(t.n, 256), 256, 0, s>>>(col, t.n, a,
                                                    (unsigned long long *) ctx->d_red);
    long long c = 0;
    ABL_CUDA_TRY(cudaMemcpyAsync(&c, ctx->d_red, sizeof c, cudaMemcpyDeviceToHost, s));
    ABL_CUDA_TRY(cudaStreamSynchronize(s));
    *(int *) out = (int) c;
    return ABL_OK;
  }
  return ABL_E_INVALID;
}

void abl_seq_record_error(abl_ctx *ctx, int code) {
  if (ctx && code != ABL_OK && ctx->seq_error == ABL_OK) ctx->seq_error = code;
}

int abl_set_seed(abl_ctx *ctx, uint64_t seed) {
  if (!ctx) return ABL_E_INVALID;
  ctx->seed = seed;
  return ABL_OK;
}

int abl_last_timestep_time(abl_ctx *ctx, double *seconds) {
  if (!ctx || !seconds) return ABL_E_INVALID;
  *seconds = ctx->last_timestep;
  return ABL_OK;
}

int abl_log_csv(abl_ctx *ctx, const char *fmt, ...) {
  if (!ctx || !fmt) return ABL_E_INVALID;
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  int len = std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (len < 0) return ABL_E_INVALID;
  ctx->log.append(buf, std::min<size_t>((size_t) len, sizeof buf - 1));
  return ABL_OK;
}

int abl_log_text(abl_ctx *ctx, char *buf, size_t cap, size_t *len) {
  if (!ctx) return ABL_E_INVALID;
  if (len) *len = ctx->log.size();
  if (buf && cap) {
    size_t c = std::min(cap - 1, ctx->log.size());
    std::memcpy(buf, ctx->log.data(), c);
    buf[c] = 0;
  }
  return ABL_OK;
}

int abl_last_exec_time(abl_ctx *ctx, double *seconds) {
  if (!ctx || !seconds) return ABL_E_INVALID;
  *seconds = ctx->last_exec;
  return ABL_OK;
}

int abl_memory_used(abl_ctx *ctx, size_t *bytes) {
  if (!ctx || !bytes) return ABL_E_INVALID;
  *bytes = ctx->used;
  return ABL_OK;
}

int abl_last_launch_count(abl_ctx *ctx, long *launches) {
  if (!ctx || !launches) return ABL_E_INVALID;
  *launches = ctx->last_launches;
  return ABL_OK;
}

int abl_set_profiling(abl_ctx *ctx, int enable) {
  if (!ctx) return ABL_E_INVALID;
  ctx->profile = enable != 0;
  size_t ns = (size_t) ctx->model->num_steps;
  ctx->prof_pending.assign(ns, {});
  ctx->prof_seconds.assign(ns, 0.0);
  ctx->prof_launches.assign(ns, 0);
  return ABL_OK;
}

int abl_set_near_mode(abl_ctx *ctx, int mode) {
  if (!ctx || mode < ABL_NEAR_AUTO || mode > ABL_NEAR_BLOCK) return ABL_E_INVALID;
  ctx->near_mode = mode;
  ctx->prepared = false;
  drop_graph(ctx);
  return ABL_OK;
}

int abl_set_near_cache(abl_ctx *ctx, int enable) {
  if (!ctx) return ABL_E_INVALID;
  ctx->near_cache = enable != 0;
  drop_graph(ctx);
  return ABL_OK;
}

int abl_set_serial_random(abl_ctx *ctx, const uint64_t *state) {
  if (!ctx) return ABL_E_INVALID;
  drop_graph(ctx);
  if (!state) {
    if (ctx->serial_rng) dev_free(ctx, ctx->serial_rng);
    ctx->serial_rng = nullptr;
    return ABL_OK;
  }
  if (!ctx->serial_rng) ABL_TRY(dev_alloc_t(ctx, &ctx->serial_rng, 2));
  ABL_CUDA_TRY(cudaMemcpyAsync(ctx->serial_rng, state, 2 * sizeof(uint64_t),
                               cudaMemcpyHostToDevice, ctx->stream));
  ABL_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return ABL_OK;
}

int abl_get_serial_random(abl_ctx *ctx, uint64_t *state) {
  if (!ctx || !state || !ctx->serial_rng) return ABL_E_INVALID;
  ABL_CUDA_TRY(cudaMemcpyAsync(state, ctx->serial_rng, 2 * sizeof(uint64_t),
                               cudaMemcpyDeviceToHost, ctx->stream));
  ABL_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return ABL_OK;
}

int abl_set_balance(abl_ctx *ctx, int enable) {
  if (!ctx) return ABL_E_INVALID;
  ctx->balance = enable != 0;
  drop_graph(ctx);
  return ABL_OK;
}

int abl_step_kernel_time(abl_ctx *ctx, int step, double *seconds, long *launches) {
  if (!ctx || step < 0 || step >= (int) ctx->prof_seconds.size()) return ABL_E_INVALID;
  if (seconds) *seconds = ctx->prof_seconds[step];
  if (launches) *launches = ctx->prof_launches[step];
  return ABL_OK;
}

int abl_destroy(abl_ctx *ctx) {
  if (!ctx) return ABL_E_INVALID;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  drop_graph(ctx);
  for (void *p : ctx->allocations) cudaFreeAsync(p, ctx->stream);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  release_error_slot(ctx->error_host);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->ts0) cudaEventDestroy(ctx->ts0);
  if (ctx->ts1) cudaEventDestroy(ctx->ts1);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return ABL_OK;
}

const char *abl_strerror(int code) {
  switch (code) {
    case ABL_OK: return "ok";
    case ABL_E_INVALID: return "invalid argument";
    case ABL_E_BUDGET: return "device memory budget exhausted";
    case ABL_E_CUDA: return "CUDA runtime error";
    case ABL_E_TIMEOUT: return "bounded device wait timed out";
    case ABL_E_NONFINITE: return "agent position is NaN or infinite";
    case ABL_E_UNSUPPORTED: return "unsupported model feature";
    case ABL_E_CAPACITY: return "agent capacity exceeded";
    case ABL_E_NOMODEL: return "unknown model";
    case ABL_E_IO: return "state file could not be written, read or matched to the model";
    case ABL_E_SCRATCH:
      return "problem larger than the fixed scratch area of abl_step_noalloc "
             "(see ABL_NOALLOC_MAX_AGENTS / ABL_NOALLOC_MAX_CELLS)";
    default: return "unknown error";
  }
}

}  // extern "C"

// ------------------------------------------------- allocation-free timestep
//
// abl_step_noalloc runs one timestep of a single-type model on device buffers
// the caller owns, for callers that cannot allocate device memory while they
// run -- code that executes inside another framework's memory pool or
// allocator, or that must not allocate once it has started (for example
// between the steps of a real-time loop).  All temporary storage (grid
// counts, the counting sort, gathered neighbour data, neighbourhood lists,
// scan partials, the error word) lives in one fixed, file-scope device array.
// Its address is looked up with cudaGetSymbolAddress once per device, on the
// first call made with that device current; that first call also builds the
// host-side bookkeeping, so it should be made before any stream capture.
// Every call shares the array: calls that overlap on the GPU race with each
// other and must be serialised by the caller.

namespace {

constexpr long kNoAllocMaxAgents = ABL_NOALLOC_MAX_AGENTS;
constexpr long kNoAllocMaxCells = ABL_NOALLOC_MAX_CELLS;
constexpr size_t kNoAllocScratchBytes = ABL_NOALLOC_SCRATCH_BYTES;
constexpr int kNoAllocDevices = 64;

}  // namespace

static __device__ __align__(256) unsigned char abl_noalloc_scratch[kNoAllocScratchBytes];

namespace {

struct NoAllocDevice {
  bool ready = false;
  unsigned char *scratch = nullptr;  // device address of abl_noalloc_scratch
  abl_ctx *ctx = nullptr;            // reusable host bookkeeping
};
NoAllocDevice g_noalloc[kNoAllocDevices];
std::mutex g_noalloc_mutex;

struct Bump {
  unsigned char *base;
  size_t used, cap;
  template <typename T>
  T *take(size_t count) {
    size_t bytes = (std::max<size_t>(count, 1) * sizeof(T) + 255) & ~(size_t) 255;
    if (used + bytes > cap) return nullptr;
    T *p = (T *) (base + used);
    used += bytes;
    return p;
  }
};

bool scan_plan_static(ScanPlan &p, long m, Bump &b) {
  p.levels.clear();
  long len = m;
  for (;;) {
    if (p.levels.size() == p.levels.capacity()) return false;  // would allocate
    ScanLevel L;
    L.m = len;
    L.nb = std::max<long>(1, (len + kScanBlock - 1) / kScanBlock);
    L.incl = b.take<int>(len);
    L.sums = b.take<int>(L.nb);
    L.offs = b.take<int>(L.nb + 1);
    if (!L.incl || !L.sums || !L.offs) return false;
    p.levels.push_back(L);
    if (L.nb == 1) return true;
    len = L.nb;
  }
}

}  // namespace

extern "C" int abl_step_noalloc(const abl_model_desc *model, const void *globals,
                                size_t globals_size, const void *const *in_cols,
                                void *const *out_cols, size_t n, void *stream) {
  if (!model || !globals || !in_cols || !out_cols) return ABL_E_INVALID;
  if (globals_size != model->globals_size) return ABL_E_INVALID;
  if (model->num_agent_types != 1 || model->num_steps != 1) return ABL_E_UNSUPPORTED;
  // A sequential step needs the context's events and reductions; removal and
  // addition resize the population (an allocation); random() is keyed by a
  // timestep and seed that this entry point does not take.  All are refused
  // before any GPU work.
  if (model->seq_step) return ABL_E_UNSUPPORTED;
  {
    const abl_step_desc &s0 = model->steps[0];
    if (s0.uses_remove || s0.add_type >= 0 || s0.uses_rng) return ABL_E_UNSUPPORTED;
    if (s0.near_members_f32 || s0.near_pos_lo) return ABL_E_UNSUPPORTED;  // mixed form
  }
  if ((long) n > kNoAllocMaxAgents) return ABL_E_SCRATCH;
  const abl_agent_desc &ad = model->agents[0];
  if (ad.num_members > ABL_MAX_MEMBERS) return ABL_E_UNSUPPORTED;
  int dev = 0;
  ABL_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocDevices) return ABL_E_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  NoAllocDevice &D = g_noalloc[dev];
  if (!D.ready) {
    // One-time set-up on this device (host bookkeeping and the device
    // address of the static scratch array).
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, abl_noalloc_scratch);
    if (e != cudaSuccess) {
      std::fprintf(stderr, "openabl-cuda: cudaGetSymbolAddress(abl_noalloc_scratch) failed: %s\n",
                   cudaGetErrorString(e));
      return ABL_E_CUDA;
    }
    D.scratch = (unsigned char *) p;
    D.ctx = new abl_ctx;
    D.ctx->globals.reserve(16384);
    D.ctx->types.resize(1);
    D.ctx->types[0].cell_scan.levels.reserve(8);
    D.ctx->types[0].nb_scan.levels.reserve(8);
    D.ctx->grids.resize(1);
    D.ctx->grid_type.assign(1, 0);
    D.ctx->step_grid.assign(1, -1);
    D.ctx->grids[0].cell_scan.levels.reserve(8);
    D.ctx->grids[0].nb_scan.levels.reserve(8);
    D.ready = true;
  }
  if (model->globals_size > D.ctx->globals.capacity()) return ABL_E_SCRATCH;

  abl_ctx &ctx = *D.ctx;
  ctx.model = model;
  ctx.stream = (cudaStream_t) stream;
  ctx.globals.assign((const unsigned char *) globals, (const unsigned char *) globals + globals_size);
  ctx.profile = false;
  ctx.near_cache = false;  // kept lists would need an allocation per binning
  ctx.skip_stores = false; // the caller's output buffers hold nothing yet
  const void *G = ctx.globals.data();
  TypeState &t = ctx.types[0];
  t.d = &ad;
  t.n = (long) n;
  t.uploaded = true;
  t.cur = 0;
  for (int k = 0; k < ad.num_members; k++) {
    t.cols[0][k] = const_cast<void *>(in_cols[k]);
    t.cols[1][k] = out_cols[k];
  }

  Bump b{D.scratch, 0, kNoAllocScratchBytes};
  ctx.error = b.take<int>(1);
  t.amax = b.take<float>(1);
  ctx.grids[0].amax = b.take<float>(1);

  // Grid of the neighbour type, as prepare() sizes it (one grid, cells just
  // wider than the near radius).
  const abl_step_desc &sd = model->steps[0];
  ctx.step_grid[0] = sd.near_type == 0 ? 0 : -1;
  ctx.grid_type[0] = 0;
  TypeState &gb = ctx.grids[0];
  gb.d = &ad;
  gb.is_near = sd.near_type == 0;
  const int depth = gb.is_near ? list_depth(sd, ad, ctx.near_mode) : 0;
  gb.ordered = depth == 2;
  gb.rows = depth == 1;
  gb.gather_mask = gb.is_near ? sd.near_members : 0;
  gb.dirty = true;
  gb.n = t.n;
  gb.cap = t.n;
  gb.cell_scan.levels.clear();
  gb.nb_scan.levels.clear();
  if (gb.is_near) {
    if (ad.position_member < 0) return ABL_E_UNSUPPORTED;
    int dim = ad.dim;
    double emin[3] = {0, 0, 0}, emax[3] = {0, 0, 0};
    if (model->env_bounds) model->env_bounds(G, emin, emax);
    double rmax = sd.radius ? sd.radius(G) : 0.0;
    if (!(rmax > 0.0) || !std::isfinite(rmax)) rmax = model->granularity ? model->granularity(G) : 0.0;
    if (!(rmax > 0.0) || !std::isfinite(rmax)) return ABL_E_INVALID;
    double cell = rmax * (1.0 + 1.0 / 1024.0);
    gb.R = 1;
    gb.inv_cell = 1.0 / cell;
    int dims[3] = {1, 1, 1};
    for (int d = 0; d < 3; d++) {
      gb.lo[d] = d < dim ? emin[d] : 0.0;
      if (d < dim) {
        double ext = emax[d] - emin[d];
        if (!(ext >= 0.0) || !std::isfinite(ext)) return ABL_E_INVALID;
        double k = std::floor(ext * gb.inv_cell) + 1.0;
        if (k > (double) kNoAllocMaxCells) return ABL_E_SCRATCH;
        dims[d] = (int) k;
      }
    }
    gb.nx = dims[0];
    gb.ny = dims[1];
    gb.nz = dims[2];
    gb.ncells = (long) gb.nx * gb.ny * gb.nz;
    if (gb.ncells > kNoAllocMaxCells) return ABL_E_SCRATCH;
    long nn = std::max<long>(t.n, 1);
    gb.cell_count = b.take<int>(gb.ncells);
    gb.cell_start = b.take<int>(gb.ncells + 1);
    gb.local_rank = b.take<int>(nn);
    gb.cell_of = b.take<int>(nn);
    gb.order = b.take<int>(nn);
    gb.posf = b.take<float>(nn * dim);
    bool ok = gb.cell_count && gb.cell_start && gb.local_rank && gb.cell_of && gb.order && gb.posf
              && scan_plan_static(gb.cell_scan, gb.ncells, b);
    for (int k = 0; k < ad.num_members && ok; k++) {
      gb.gcols[k] = nullptr;
      if (gb.gather_mask & (1u << k)) {
        gb.gcols[k] = b.take<unsigned char>(member_bytes(ad.members[k]) * nn);
        ok = gb.gcols[k] != nullptr;
      }
    }
    gb.sep = SepLevels();
    gb.nb_off = gb.nb_list = nullptr;
    if (ok && (gb.ordered || gb.rows)) {
      long span = 2 * gb.R + 1, level = nn;
      const int inter = gb.ordered ? dim - 1 : 1;
      for (int a = 0; a < inter && ok; a++) {
        level *= span;
        gb.sep.off[a] = b.take<int>(gb.ncells + 1);
        gb.sep.elem[a] = b.take<int4>(level);
        ok = gb.sep.off[a] && gb.sep.elem[a];
      }
      gb.nb_cnt = b.take<int>(gb.ncells);
      ok = ok && gb.nb_cnt && scan_plan_static(gb.nb_scan, gb.ncells, b);
      if (ok && gb.ordered) {
        gb.nb_off = b.take<int>(gb.ncells + 1);
        gb.nb_list = b.take<int>(level * span);
        ok = gb.nb_off && gb.nb_list;
      }
    }
    if (!ok) return ABL_E_SCRATCH;
  }
  ctx.prepared = true;

  // The scratch keeps the previous call's contents: clear the words that
  // must start at zero (the cell counters are cleared by the binning itself).
  ABL_CUDA_TRY(cudaMemsetAsync(ctx.error, 0, sizeof(int), ctx.stream));
  ABL_CUDA_TRY(cudaMemsetAsync(t.amax, 0, sizeof(float), ctx.stream));
  if (t.n > 0) ABL_TRY(step_once(&ctx));
  int h = 0;
  ABL_CUDA_TRY(cudaMemcpyAsync(&h, ctx.error, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
  ABL_CUDA_TRY(cudaStreamSynchronize(ctx.stream));
  return h;
}

// ------------------------------------------------------------- ensembles
//
// An ensemble runs many replicas of one model -- different agent counts,
// different globals (parameter points), different random seeds -- as one
// population.  Replica r's agents of a type occupy [base[r], base[r] +
// count[r]) of shared columns; each replica has its own grid, and the grids
// are laid end to end in one cell array (a segmented grid), so binning, the
// prefix scans, the neighbourhood lists and every step function run as ONE
// launch over all replicas.  Two timesteps are captured into a CUDA graph and
// replayed.  Results are per replica what a separate context would compute:
// step kernels read the replica's globals and grid view, slots and cell
// starts are global, and random() is keyed by the replica's seed and the
// agent's index within its replica.

namespace {

template <typename Real, int DIM>
__global__ void k_ens_bin_assign(const Real *pos, long n, const int *replica_of,
                                 const EnsGrid *grids, int *cell_of, int *cell_count,
                                 int *local_rank, float *amax, int *error) {
  long i = (long) blockIdx.x * blockDim.x + threadIdx.x;
  float m = 0.0f;
  if (i < n)
    m = ens_bin_assign_item<Real, DIM>(i, pos, replica_of, grids, cell_of, cell_count,
                                       local_rank, error);
  fold_amax(m, amax);
}


struct EnsType {
  const abl_agent_desc *d = nullptr;
  long n = 0;
  std::vector<long> counts, base;
  void *cols[2][ABL_MAX_MEMBERS] = {};
  int cur = 0;
  int *replica_of = nullptr;
  long *d_base = nullptr;
  bool uploaded = false;
  // binning
  bool is_near = false, ordered = false, rows = false, dirty = true;
  uint32_t gather_mask = 0;
  std::vector<EnsGrid> grids;
  EnsGrid *d_grids = nullptr;
  long ncells = 0;
  int *cell_replica = nullptr;
  int *cell_count = nullptr, *cell_start = nullptr, *local_rank = nullptr, *cell_of = nullptr;
  int *order = nullptr;
  float *posf = nullptr, *amax = nullptr;
  float *amax_acc = nullptr;  // persistent runs: the assign phase's maximum
  void *gcols[ABL_MAX_MEMBERS] = {};
  int *nb_cnt = nullptr, *nb_off = nullptr, *nb_list = nullptr;
  SepLevels sep;
  ScanPlan cell_scan, nb_scan;
  std::vector<void *> allocs;
};

}  // namespace

struct abl_ensemble {
  abl_ctx base;  // stream, allocations, budget, scans
  int replicas = 0;
  std::vector<unsigned char> globals;  // replicas x globals_size
  void *d_globals = nullptr;
  uint64_t *d_seeds = nullptr;
  std::vector<uint64_t> seeds;
  std::vector<EnsType> types;
  std::vector<abl_near_view *> d_views;  // per step with a near loop
  std::vector<void *> view_allocs;
  bool prepared = false;
  int block = 128;
  double cell_factor = 1.0;
  int visit_sorted = 1;
  int balance = 1;
  std::vector<size_t> smem;  // per step: dynamic shared memory of its kernel
  std::vector<abl_ctx::Graph> graphs;
  long timestep = 0;
  // persistent runs (abl_ensemble_set_persistent)
  bool persistent = false;
  abl::persist_prog *d_prog = nullptr;
  abl::persist_sync *d_sync = nullptr;
  unsigned long long *d_stamps = nullptr;  // phase end times of the last run's first phases
  unsigned long long barrier_limit_ns = 4000000000ull;
  unsigned int barrier_extra = 0;
  int persist_grid = 0;
};

namespace {

void ens_free_bins(abl_ensemble *e, EnsType &t) {
  for (void *p : t.allocs) dev_free(&e->base, p);
  t.allocs.clear();
  t.cell_scan.levels.clear();
  t.nb_scan.levels.clear();
  t.cell_count = t.cell_start = t.local_rank = t.cell_of = t.order = nullptr;
  t.nb_cnt = t.nb_off = t.nb_list = t.cell_replica = nullptr;
  t.sep = SepLevels();
  t.posf = t.amax = t.amax_acc = nullptr;
  t.d_grids = nullptr;
  for (auto &g : t.gcols) g = nullptr;
}

void ens_drop_graphs(abl_ensemble *e) {
  for (auto &g : e->graphs) cudaGraphExecDestroy(g.exec);
  e->graphs.clear();
}

int ens_prepare(abl_ensemble *e) {
  abl_ctx *ctx = &e->base;
  const abl_model_desc *m = ctx->model;
  ens_drop_graphs(e);
  for (void *p : e->view_allocs) dev_free(ctx, p);
  e->view_allocs.clear();
  e->d_views.assign(m->num_steps, nullptr);
  e->smem.assign(m->num_steps, 0);
  for (int ti = 0; ti < m->num_agent_types; ti++) {
    EnsType &t = e->types[ti];
    ens_free_bins(e, t);
    t.is_near = false;
    t.ordered = false;
    t.rows = false;
    t.gather_mask = 0;
    for (int k = 0; k < m->num_steps; k++) {
      const abl_step_desc &sd = m->steps[k];
      if (sd.near_type != ti) continue;
      t.is_near = true;
      const int depth = list_depth(sd, *t.d, ctx->near_mode);
      t.ordered = t.ordered || depth == 2;
      t.rows = t.rows || depth == 1;
      t.gather_mask |= sd.near_members;
    }
    auto *own = &t.allocs;
    ABL_TRY(dev_alloc_t(ctx, &t.amax, 1, own));
    ABL_TRY(dev_alloc_t(ctx, &t.amax_acc, 1, own));
    if (!t.is_near) continue;
    int dim = t.d->dim;
    t.grids.assign(e->replicas, EnsGrid());
    long cells = 0;
    for (int r = 0; r < e->replicas; r++) {
      const void *G = e->globals.data() + (size_t) r * m->globals_size;
      double emin[3] = {0, 0, 0}, emax[3] = {0, 0, 0};
      if (m->env_bounds) m->env_bounds(G, emin, emax);
      double rmax = 0.0;
      for (int k = 0; k < m->num_steps; k++) {
        if (m->steps[k].near_type == ti && m->steps[k].radius)
          rmax = std::max(rmax, m->steps[k].radius(G));
      }
      double gran = m->granularity ? m->granularity(G) : rmax;
      if (!(gran > 0.0) || !std::isfinite(gran)) return ABL_E_INVALID;
      double cell = gran * (1.0 + 1.0 / 1024.0) * std::max(1.0, e->cell_factor);
      EnsGrid &g = t.grids[r];
      g.R = std::max(1, (int) std::ceil(rmax * (1.0 + 1e-6) / cell));
      if (2 * g.R + 1 > kSepMaxSrc) return ABL_E_UNSUPPORTED;
      g.inv_cell = 1.0 / cell;
      int dims[3] = {1, 1, 1};
      for (int d = 0; d < 3; d++) {
        g.lo[d] = d < dim ? emin[d] : 0.0;
        if (d < dim) {
          double ext = emax[d] - emin[d];
          if (!(ext >= 0.0) || !std::isfinite(ext)) return ABL_E_INVALID;
          double k = std::floor(ext * g.inv_cell) + 1.0;
          if (k > 1 << 24) return ABL_E_UNSUPPORTED;
          dims[d] = (int) k;
        }
      }
      g.nx = dims[0];
      g.ny = dims[1];
      g.nz = dims[2];
      // FP32 cell coordinates where the rounding-error bound allows them
      // (the radius prefilter decides the same neighbours either way; only
      // the FP64 pipe's load changes).
      g.f32 = fp32_cells_ok(g.lo, g.inv_cell, dims, dim) ? 1 : 0;
      for (int d = 0; d < 3; d++) g.flo[d] = (float) g.lo[d];
      g.finv = (float) g.inv_cell;
      g.cell_base = cells;
      cells += (long) g.nx * g.ny * g.nz;
      if (cells > (1L << 30)) return ABL_E_UNSUPPORTED;
    }
    t.ncells = cells;
    long n = std::max<long>(t.n, 1);
    ABL_TRY(dev_alloc_t(ctx, &t.d_grids, e->replicas, own));
    ABL_CUDA_TRY(cudaMemcpy(t.d_grids, t.grids.data(), sizeof(EnsGrid) * e->replicas,
                            cudaMemcpyHostToDevice));
    std::vector<int> cr(cells);
    for (int r = 0; r < e->replicas; r++) {
      long c0 = t.grids[r].cell_base;
      long c1 = r + 1 < e->replicas ? t.grids[r + 1].cell_base : cells;
      for (long c = c0; c < c1; c++) cr[c] = r;
    }
    ABL_TRY(dev_alloc_t(ctx, &t.cell_replica, std::max<long>(cells, 1), own));
    ABL_CUDA_TRY(cudaMemcpy(t.cell_replica, cr.data(), sizeof(int) * cells,
                            cudaMemcpyHostToDevice));
    ABL_TRY(dev_alloc_t(ctx, &t.cell_count, cells, own));
    ABL_TRY(dev_alloc_t(ctx, &t.cell_start, cells + 1, own));
    ABL_TRY(dev_alloc_t(ctx, &t.local_rank, n, own));
    ABL_TRY(dev_alloc_t(ctx, &t.cell_of, n, own));
    ABL_TRY(dev_alloc_t(ctx, &t.order, n, own));
    ABL_TRY(dev_alloc_t(ctx, &t.posf, n * dim, own));
    ABL_TRY(scan_plan(ctx, t.cell_scan, cells, own));
    for (int k = 0; k < t.d->num_members; k++) {
      if (t.gather_mask & (1u << k)) {
        void *p = nullptr;
        ABL_TRY(dev_alloc(ctx, &p, member_bytes(t.d->members[k]) * n, own));
        t.gcols[k] = p;
      }
    }
    if (t.ordered || t.rows) {
      int Rmax = 1;
      for (auto &g : t.grids) Rmax = std::max(Rmax, g.R);
      long span = 2 * Rmax + 1, level = n;
      const int inter = t.ordered ? dim - 1 : 1;
      for (int a = 0; a < inter; a++) {
        level *= span;
        ABL_TRY(dev_alloc_t(ctx, &t.sep.off[a], cells + 1, own));
        ABL_TRY(dev_alloc_t(ctx, &t.sep.elem[a], level, own));
      }
      if (level * (t.ordered ? span : 1) > (long) INT32_MAX) return ABL_E_UNSUPPORTED;
      ABL_TRY(dev_alloc_t(ctx, &t.nb_cnt, cells, own));
      ABL_TRY(scan_plan(ctx, t.nb_scan, cells, own));
      if (t.ordered) {
        ABL_TRY(dev_alloc_t(ctx, &t.nb_off, cells + 1, own));
        ABL_TRY(dev_alloc_t(ctx, &t.nb_list, level * span, own));
      }
    }
    t.dirty = true;
  }
  // Per replica neighbour views for every step function with a near loop.
  for (int k = 0; k < m->num_steps; k++) {
    const abl_step_desc &sd = m->steps[k];
    if (sd.near_type < 0) continue;
    EnsType &nt = e->types[sd.near_type];
    std::vector<abl_near_view> views(e->replicas);
    for (int r = 0; r < e->replicas; r++) {
      const EnsGrid &g = nt.grids[r];
      abl_near_view &V = views[r];
      std::memset(&V, 0, sizeof V);
      const int depth = list_depth(sd, *nt.d, ctx->near_mode);
      V.dim = nt.d->dim;
      V.ordered = depth == 2;
      V.rows = depth == 1 ? nt.sep.elem[0] : nullptr;
      V.row_off = nt.sep.off[0] ? nt.sep.off[0] + g.cell_base : nullptr;
      V.range = g.R;
      V.nx = g.nx;
      V.ny = g.ny;
      V.nz = g.nz;
      for (int d = 0; d < 3; d++) V.lo[d] = g.lo[d];
      V.inv_cell = g.inv_cell;
      V.cell_f32 = g.f32;
      V.radius = sd.radius(e->globals.data() + (size_t) r * m->globals_size);
      V.n = nt.counts.empty() ? 0 : nt.counts[r];
      V.cell_start = nt.cell_start + g.cell_base;
      V.order = nt.order;
      V.posf = nt.posf;
      V.nb_off = nt.nb_off ? nt.nb_off + g.cell_base : nullptr;
      V.nb_list = nt.nb_list;
      V.amax = nt.amax;
      for (int j = 0; j < nt.d->num_members; j++) V.cols[j] = nt.gcols[j];
      V.balance = e->balance;
      V.cap = V.ordered ? ctx->list_cap : ctx->runs_cap;
      V.cell_of = sd.agent_type == sd.near_type ? nt.cell_of : nullptr;
      V.cell_base = g.cell_base;
      V.block_cap = e->visit_sorted && block_lists_wanted(sd, depth, ctx->near_mode)
                        ? ctx->block_cap : 0;
    }
    e->smem[k] = sd.presorted ? abl::presort_bytes(views[0]) : 0;
    abl_near_view *dv = nullptr;
    ABL_TRY(dev_alloc_t(ctx, &dv, views.size(), &e->view_allocs));
    ABL_CUDA_TRY(cudaMemcpy(dv, views.data(), sizeof(abl_near_view) * views.size(),
                            cudaMemcpyHostToDevice));
    e->d_views[k] = dv;
  }
  e->prepared = true;
  return ABL_OK;
}

template <typename Real>
void ens_launch_bin(abl_ensemble *e, EnsType &t) {
  abl_ctx *ctx = &e->base;
  cudaStream_t s = ctx->stream;
  const int B = 256;
  int dim = t.d->dim;
  long nb = blocks_for(t.n, B);
  const Real *pos = (const Real *) t.cols[t.cur][t.d->position_member];
  cudaMemsetAsync(t.cell_count, 0, sizeof(int) * t.ncells, s);
  cudaMemsetAsync(t.amax, 0, sizeof(float), s);
  if (dim == 2) {
    k_ens_bin_assign<Real, 2><<<nb, B, 0, s>>>(pos, t.n, t.replica_of, t.d_grids, t.cell_of,
                                               t.cell_count, t.local_rank, t.amax, ctx->error);
  } else {
    k_ens_bin_assign<Real, 3><<<nb, B, 0, s>>>(pos, t.n, t.replica_of, t.d_grids, t.cell_of,
                                               t.cell_count, t.local_rank, t.amax, ctx->error);
  }
  ctx->launches++;
  scan_run(ctx, t.cell_scan, t.cell_count, t.cell_start);
  k_bin_scatter<<<nb, B, 0, s>>>(t.n, t.cell_of, t.local_rank, t.cell_start, t.order);
  ctx->launches++;
  k_cell_sort<<<blocks_for(t.ncells, B), B, 0, s>>>(t.ncells, t.cell_start, t.order);
  ctx->launches++;
  GatherArgs g;
  std::memset(&g, 0, sizeof g);
  for (int k = 0; k < t.d->num_members; k++) {
    if (!(t.gather_mask & (1u << k))) continue;
    g.src[g.nmem] = t.cols[t.cur][k];
    g.dst[g.nmem] = t.gcols[k];
    g.bytes[g.nmem] = (int) member_bytes(t.d->members[k]);
    g.nmem++;
  }
  if (dim == 2) k_gather<Real, 2><<<nb, B, 0, s>>>(t.n, t.order, pos, t.posf, g);
  else k_gather<Real, 3><<<nb, B, 0, s>>>(t.n, t.order, pos, t.posf, g);
  ctx->launches++;
  if (t.ordered || t.rows) {
    int Rmax = 1;
    for (auto &g : t.grids) Rmax = std::max(Rmax, g.R);
    EnsGeom geo{t.cell_replica, t.d_grids};
    build_lists(ctx, geo, dim, t.ordered ? dim : 1, Rmax, t.ncells, t.cell_start, t.order,
                t.posf, t.sep, t.nb_cnt, t.nb_scan, t.nb_off, t.nb_list);
  }
  t.dirty = false;
}

int ens_step_once(abl_ensemble *e) {
  abl_ctx *ctx = &e->base;
  const abl_model_desc *m = ctx->model;
  for (int k = 0; k < m->num_steps; k++) {
    const abl_step_desc &sd = m->steps[k];
    EnsType &t = e->types[sd.agent_type];
    if (sd.near_type >= 0) {
      EnsType &nt = e->types[sd.near_type];
      if (nt.dirty) {
        if (nt.d->members[nt.d->position_member].scalar_bytes == 8)
          ens_launch_bin<double>(e, nt);
        else
          ens_launch_bin<float>(e, nt);
      }
    }
    abl_ens_launch L;
    std::memset(&L, 0, sizeof L);
    L.n = t.n;
    for (int j = 0; j < t.d->num_members; j++) {
      L.in_cols[j] = t.cols[t.cur][j];
      L.out_cols[j] = t.cols[1 - t.cur][j];
    }
    L.visit_order = (e->visit_sorted && sd.near_type == sd.agent_type) ? t.order : nullptr;
    L.replica = t.replica_of;
    L.globals = e->d_globals;
    L.views = sd.near_type >= 0 ? e->d_views[k] : nullptr;
    L.smem = e->smem[k];
    L.agent_base = t.d_base;
    L.seeds = e->d_seeds;
    L.timestep = e->timestep;
    L.step_index = k;
    L.block = e->block;
    if (t.n > 0) {
      ABL_TRY(sd.launch_ens(&L, ctx->stream));
      ctx->launches++;
    }
    t.cur = 1 - t.cur;
    t.dirty = true;
  }
  e->timestep++;
  return ABL_OK;
}

std::vector<int> ens_graph_key(const abl_ensemble *e) {
  std::vector<int> key;
  for (const EnsType &t : e->types) {
    key.push_back(t.cur);
    key.push_back(t.dirty ? 1 : 0);
  }
  return key;
}

int ens_capture(abl_ensemble *e, abl_ctx::Graph **out) {
  std::vector<int> key = ens_graph_key(e);
  for (auto &g : e->graphs) {
    if (g.key == key) {
      *out = &g;
      return ABL_OK;
    }
  }
  abl_ctx *ctx = &e->base;
  abl_ctx::Graph G;
  G.key = key;
  long before = ctx->launches;
  long ts = e->timestep;
  cudaGraph_t g = nullptr;
  ABL_CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  int r = ens_step_once(e);
  if (r == ABL_OK) r = ens_step_once(e);
  cudaError_t err = cudaStreamEndCapture(ctx->stream, &g);
  if (r != ABL_OK) {
    if (g) cudaGraphDestroy(g);
    return r;
  }
  ABL_CUDA_TRY(err);
  err = cudaGraphInstantiate(&G.exec, g, 0);
  cudaGraphDestroy(g);
  ABL_CUDA_TRY(err);
  G.launches = ctx->launches - before;
  ctx->launches = before;
  e->timestep = ts;
  for (size_t k = 0; k < e->types.size(); k++) {
    e->types[k].cur = key[2 * k];
    e->types[k].dirty = key[2 * k + 1] != 0;
  }
  e->graphs.push_back(G);
  *out = &e->graphs.back();
  return ABL_OK;
}

// ---------------------------------------------------- persistent runs
//
// A persistent run records the ops of a timestep -- the binnings and step
// functions ens_step_once would launch, with the buffers they would use --
// into a program (abl_persist.cuh) and runs all timesteps in one cooperative
// launch of the model's persistent kernel.  The double buffers flip every
// timestep, so from the second timestep on the program repeats with period
// two; the first may differ (types that are binned once and never stepped).

// Phase end times a persistent run records (block 0, after each barrier).
constexpr int kPersistStamps = 64;

// The binning of `t` from its current buffer, as ens_launch_bin does it.
void ens_persist_bin(abl_ensemble *e, EnsType &t, abl::persist_bin &B) {
  std::memset(&B, 0, sizeof B);
  const int dim = t.d->dim;
  B.dim = dim;
  B.pos_double = t.d->members[t.d->position_member].scalar_bytes == 8;
  B.n = t.n;
  B.ncells = t.ncells;
  B.pos = t.cols[t.cur][t.d->position_member];
  B.replica_of = t.replica_of;
  B.grids = t.d_grids;
  B.cell_replica = t.cell_replica;
  B.cell_of = t.cell_of;
  B.cell_count = t.cell_count;
  B.local_rank = t.local_rank;
  B.order = t.order;
  B.cell_start = t.cell_start;
  B.posf = t.posf;
  B.amax = t.amax;
  B.amax_acc = t.amax_acc;
  // Chunks of kScanBlock ints: the scan plan's first level has the room.
  B.scan_incl = t.cell_scan.levels[0].incl;
  B.scan_sums = t.cell_scan.levels[0].sums;
  for (int k = 0; k < t.d->num_members; k++) {
    if (!(t.gather_mask & (1u << k))) continue;
    GatherArgs &g = B.gather;
    g.src[g.nmem] = t.cols[t.cur][k];
    g.dst[g.nmem] = t.gcols[k];
    g.bytes[g.nmem] = (int) member_bytes(t.d->members[k]);
    g.nmem++;
  }
  if (t.ordered || t.rows) {
    B.levels = t.ordered ? dim : 1;
    B.Rmax = 1;
    for (auto &g : t.grids) B.Rmax = std::max(B.Rmax, g.R);
    B.cnt = t.nb_cnt;
    for (int a = 0; a < B.levels; a++) {
      const bool last = a == dim - 1;
      B.dst_off[a] = last ? t.nb_off : t.sep.off[a];
      B.dst_elem[a] = last ? nullptr : t.sep.elem[a];
      B.dst_slot[a] = last ? t.nb_list : nullptr;
    }
  }
}

// One timestep's ops into T (T == nullptr: only the bookkeeping -- buffer
// flips, dirty flags, timestep -- that running it leaves behind).
int ens_record(abl_ensemble *e, abl::persist_timestep *T) {
  abl_ctx *ctx = &e->base;
  const abl_model_desc *m = ctx->model;
  int nops = 0;
  auto next = [&]() -> abl::persist_op * {
    if (!T) return nullptr;
    if (nops >= abl::kPersistMaxOps) return nullptr;
    return &T->ops[nops++];
  };
  for (int k = 0; k < m->num_steps; k++) {
    const abl_step_desc &sd = m->steps[k];
    EnsType &t = e->types[sd.agent_type];
    if (sd.near_type >= 0) {
      EnsType &nt = e->types[sd.near_type];
      if (nt.dirty) {
        if (T) {
          abl::persist_op *op = next();
          if (!op) return ABL_E_UNSUPPORTED;
          op->kind = abl::kPersistBin;
          ens_persist_bin(e, nt, op->bin);
        }
        nt.dirty = false;
      }
    }
    if (T) {
      abl::persist_op *op = next();
      if (!op) return ABL_E_UNSUPPORTED;
      op->kind = abl::kPersistStep;
      abl_ens_launch &L = op->step;
      std::memset(&L, 0, sizeof L);
      L.n = t.n;
      for (int j = 0; j < t.d->num_members; j++) {
        L.in_cols[j] = t.cols[t.cur][j];
        L.out_cols[j] = t.cols[1 - t.cur][j];
      }
      L.visit_order = (e->visit_sorted && sd.near_type == sd.agent_type) ? t.order : nullptr;
      L.replica = t.replica_of;
      L.globals = e->d_globals;
      L.views = sd.near_type >= 0 ? e->d_views[k] : nullptr;
      L.smem = e->smem[k];
      L.agent_base = t.d_base;
      L.seeds = e->d_seeds;
      L.timestep = e->timestep;
      L.step_index = k;
      L.block = e->block;
    }
    t.cur = 1 - t.cur;
    t.dirty = true;
  }
  if (T) T->nops = nops;
  e->timestep++;
  return ABL_OK;
}

// Puts the bookkeeping back to `key` (ens_graph_key) and timestep `ts`.
void ens_restore(abl_ensemble *e, const std::vector<int> &key, long ts) {
  for (size_t k = 0; k < e->types.size(); k++) {
    e->types[k].cur = key[2 * k];
    e->types[k].dirty = key[2 * k + 1] != 0;
  }
  e->timestep = ts;
}

std::vector<int> ens_graph_key(const abl_ensemble *e);

int ens_run_persistent(abl_ensemble *e, int timesteps) {
  abl_ctx *ctx = &e->base;
  const abl_model_desc *m = ctx->model;
  if (!m->launch_ens_persist) return ABL_E_UNSUPPORTED;
  if (timesteps <= 0) return ABL_OK;
  if (!e->d_prog) {
    ABL_TRY(dev_alloc_t(ctx, &e->d_prog, 1));
    ABL_TRY(dev_alloc_t(ctx, &e->d_sync, 1));
    ABL_TRY(dev_alloc_t(ctx, &e->d_stamps, kPersistStamps));
  }
  std::unique_ptr<abl::persist_prog> P(new abl::persist_prog());
  const std::vector<int> k0 = ens_graph_key(e);
  const long ts0 = e->timestep;
  int r = ens_record(e, &P->ts[0]);
  const std::vector<int> k1 = ens_graph_key(e);
  if (r == ABL_OK) r = ens_record(e, &P->ts[1]);
  if (r == ABL_OK && ens_graph_key(e) != k0) {
    // The first timestep differs: ts[0] once, then ts[1], ts[2] in turn.
    P->first_special = 1;
    r = ens_record(e, &P->ts[2]);
    if (r == ABL_OK && ens_graph_key(e) != k1) r = ABL_E_UNSUPPORTED;
  }
  ens_restore(e, k0, ts0);
  if (r != ABL_OK) return r;
  size_t smem = 0;
  int levels = 0;
  for (int k = 0; k < 3; k++) {
    for (int o = 0; o < P->ts[k].nops; o++) {
      const abl::persist_op &op = P->ts[k].ops[o];
      if (op.kind == abl::kPersistStep) smem = std::max(smem, op.step.smem);
      else levels = std::max(levels, op.bin.levels);
    }
  }
  if (levels > 1)  // warp merges stage kSepStage ids per warp
    smem = std::max(smem, (size_t) (e->block / 32) * kSepStage * sizeof(int));
  P->timesteps = timesteps;
  P->base_timestep = ts0;
  P->sync = e->d_sync;
  P->limit_ns = e->barrier_limit_ns;
  P->extra_arrivals = e->barrier_extra;
  P->scan_chunk = kScanBlock;
  P->stamps = e->d_stamps;
  P->stamp_cap = kPersistStamps;
  ABL_CUDA_TRY(cudaMemsetAsync(e->d_stamps, 0, sizeof(unsigned long long) * kPersistStamps,
                               ctx->stream));
  ABL_CUDA_TRY(cudaMemcpyAsync(e->d_prog, P.get(), sizeof(abl::persist_prog),
                               cudaMemcpyHostToDevice, ctx->stream));
  ABL_CUDA_TRY(cudaMemsetAsync(e->d_sync, 0, sizeof(abl::persist_sync), ctx->stream));
  // Enough blocks for the largest step phase's virtual blocks, at least one
  // per SM (the binning phases stride over agents and cells).
  long most = 0;
  for (const EnsType &t : e->types) most = std::max(most, t.n);
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  e->persist_grid = (int) std::min<long>(1L << 30, std::max<long>(std::max(sms, 1),
                                                                   blocks_for(most, e->block)));
  ABL_TRY(m->launch_ens_persist(e->d_prog, ctx->error, e->block, smem, &e->persist_grid,
                                ctx->stream));
  ctx->launches++;
  // The host copy of the program must outlive the asynchronous copy.
  ABL_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  for (int it = 0; it < timesteps; it++) ens_record(e, nullptr);
  return ABL_OK;
}

// The barrier's error word after a persistent run (0 or ABL_E_TIMEOUT).
int ens_persist_error(abl_ensemble *e) {
  if (!e->d_sync) return ABL_OK;
  int h = 0;
  ABL_CUDA_TRY(cudaMemcpy(&h, &e->d_sync->error, sizeof(int), cudaMemcpyDeviceToHost));
  return h;
}

// Graph replay bakes the timestep into kernel arguments, and random() keys
// on it: models that draw in step functions run eagerly.
bool uses_rng(const abl_model_desc *m) {
  for (int k = 0; k < m->num_steps; k++)
    if (m->steps[k].uses_rng) return true;
  return false;
}

}  // namespace

extern "C" {

int abl_ensemble_create(const abl_model_desc *model, int replicas, const void *globals,
                        const uint64_t *seeds, size_t hbm_budget, abl_ensemble **out) {
  if (!model || replicas <= 0 || !out) return ABL_E_INVALID;
  if (model->seq_step) return ABL_E_UNSUPPORTED;
  for (int k = 0; k < model->num_steps; k++) {
    if (!model->steps[k].launch_ens) return ABL_E_UNSUPPORTED;
  }
  abl_ensemble *e = new abl_ensemble;
  abl_ctx *ctx = &e->base;
  ctx->model = model;
  ctx->budget = hbm_budget;
  e->replicas = replicas;
  size_t gs = model->globals_size;
  e->globals.resize(gs * replicas);
  for (int r = 0; r < replicas; r++) {
    std::memcpy(e->globals.data() + gs * r,
                globals ? (const unsigned char *) globals + gs * r
                        : (const unsigned char *) model->globals_default, gs);
  }
  e->seeds.assign(replicas, 0);
  if (seeds) e->seeds.assign(seeds, seeds + replicas);
  e->types.resize(model->num_agent_types);
  for (int k = 0; k < model->num_agent_types; k++) {
    e->types[k].d = &model->agents[k];
    e->types[k].counts.assign(replicas, 0);
    e->types[k].base.assign(replicas, 0);
  }
  cudaError_t err = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (err == cudaSuccess) err = cudaEventCreate(&ctx->ev0);
  if (err == cudaSuccess) err = cudaEventCreate(&ctx->ev1);
  if (err != cudaSuccess) {
    delete e;
    return ABL_E_CUDA;
  }
  int r = dev_alloc_t(ctx, &ctx->error, 1);
  if (r == ABL_OK) r = dev_alloc(ctx, &e->d_globals, gs * replicas);
  if (r == ABL_OK) r = dev_alloc_t(ctx, &e->d_seeds, replicas);
  if (r == ABL_OK) {
    cudaMemset(ctx->error, 0, sizeof(int));
    cudaMemcpy(e->d_globals, e->globals.data(), gs * replicas, cudaMemcpyHostToDevice);
    cudaMemcpy(e->d_seeds, e->seeds.data(), sizeof(uint64_t) * replicas, cudaMemcpyHostToDevice);
  }
  if (r != ABL_OK) {
    abl_ensemble_destroy(e);
    return r;
  }
  *out = e;
  return ABL_OK;
}

int abl_ensemble_upload(abl_ensemble *e, int type_id, const size_t *counts,
                        const void *const *cols) {
  if (!e || !counts || type_id < 0 || type_id >= (int) e->types.size()) return ABL_E_INVALID;
  abl_ctx *ctx = &e->base;
  EnsType &t = e->types[type_id];
  long total = 0;
  for (int r = 0; r < e->replicas; r++) {
    t.counts[r] = (long) counts[r];
    t.base[r] = total;
    total += (long) counts[r];
  }
  if (total > (long) INT32_MAX) return ABL_E_UNSUPPORTED;
  for (int b = 0; b < 2; b++) {
    for (int k = 0; k < t.d->num_members; k++) {
      if (t.cols[b][k]) dev_free(ctx, t.cols[b][k]);
      t.cols[b][k] = nullptr;
      ABL_TRY(dev_alloc(ctx, &t.cols[b][k], member_bytes(t.d->members[k]) * std::max<long>(total, 1)));
    }
  }
  if (t.replica_of) dev_free(ctx, t.replica_of);
  if (t.d_base) dev_free(ctx, t.d_base);
  ABL_TRY(dev_alloc_t(ctx, &t.replica_of, std::max<long>(total, 1)));
  ABL_TRY(dev_alloc_t(ctx, &t.d_base, e->replicas));
  std::vector<int> rep(total);
  for (int r = 0; r < e->replicas; r++)
    for (long i = 0; i < t.counts[r]; i++) rep[t.base[r] + i] = r;
  ABL_CUDA_TRY(cudaMemcpy(t.replica_of, rep.data(), sizeof(int) * total, cudaMemcpyHostToDevice));
  ABL_CUDA_TRY(cudaMemcpy(t.d_base, t.base.data(), sizeof(long) * e->replicas,
                          cudaMemcpyHostToDevice));
  t.n = total;
  t.cur = 0;
  for (int k = 0; k < t.d->num_members; k++) {
    size_t bytes = member_bytes(t.d->members[k]) * total;
    if (!bytes) continue;
    if (!cols || !cols[k]) return ABL_E_INVALID;
    ABL_CUDA_TRY(cudaMemcpy(t.cols[0][k], cols[k], bytes, cudaMemcpyHostToDevice));
    ABL_CUDA_TRY(cudaMemcpy(t.cols[1][k], t.cols[0][k], bytes, cudaMemcpyDeviceToDevice));
  }
  t.uploaded = true;
  t.dirty = true;
  e->prepared = false;
  e->timestep = 0;
  return ABL_OK;
}

static int ens_ready(abl_ensemble *e) {
  for (auto &t : e->types) {
    if (!t.uploaded) {
      std::vector<size_t> zero(e->replicas, 0);
      ABL_TRY(abl_ensemble_upload(e, (int) (&t - &e->types[0]), zero.data(), nullptr));
    }
  }
  if (!e->prepared) ABL_TRY(ens_prepare(e));
  return ABL_OK;
}

int abl_ensemble_run(abl_ensemble *e, int timesteps) {
  if (!e || timesteps < 0) return ABL_E_INVALID;
  ABL_TRY(ens_ready(e));
  abl_ctx *ctx = &e->base;
  long l0 = ctx->launches;
  ABL_CUDA_TRY(cudaEventRecord(ctx->ev0, ctx->stream));
  int done = 0;
  if (e->persistent && timesteps > 0) {
    ABL_TRY(ens_run_persistent(e, timesteps));
    done = timesteps;
  }
  if (done < timesteps) {
    ABL_TRY(ens_step_once(e));
    done = 1;
  }
  if (timesteps - done >= 2 && !uses_rng(ctx->model)) {
    abl_ctx::Graph *G = nullptr;
    ABL_TRY(ens_capture(e, &G));
    for (; done + 2 <= timesteps; done += 2) {
      ABL_CUDA_TRY(cudaGraphLaunch(G->exec, ctx->stream));
      ctx->launches += G->launches;
      e->timestep += 2;
    }
  }
  for (; done < timesteps; done++) ABL_TRY(ens_step_once(e));
  ABL_CUDA_TRY(cudaEventRecord(ctx->ev1, ctx->stream));
  int r = check_error(ctx);
  if (r == ABL_OK && e->persistent) r = ens_persist_error(e);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  ctx->last_exec = ms / 1000.0;
  ctx->last_launches = ctx->launches - l0;
  return r;
}

int abl_ensemble_download(abl_ensemble *e, int type_id, size_t *counts, void *const *cols) {
  if (!e || type_id < 0 || type_id >= (int) e->types.size()) return ABL_E_INVALID;
  EnsType &t = e->types[type_id];
  if (counts)
    for (int r = 0; r < e->replicas; r++) counts[r] = (size_t) t.counts[r];
  if (!cols) return ABL_OK;
  for (int k = 0; k < t.d->num_members; k++) {
    size_t bytes = member_bytes(t.d->members[k]) * t.n;
    if (!bytes) continue;
    if (!cols[k]) return ABL_E_INVALID;
    ABL_CUDA_TRY(cudaMemcpyAsync(cols[k], t.cols[t.cur][k], bytes, cudaMemcpyDeviceToHost,
                                 e->base.stream));
  }
  return check_error(&e->base);
}

int abl_ensemble_set_tuning(abl_ensemble *e, int block, double cell_factor, int visit_sorted) {
  if (!e || block <= 0 || block > ABL_STEP_BLOCK || block % 32 || !(cell_factor >= 1.0))
    return ABL_E_INVALID;
  e->block = block;
  // The views depend on both (cell sizes; block lists need slot-ordered visits).
  if (cell_factor != e->cell_factor || (visit_sorted ? 1 : 0) != e->visit_sorted)
    e->prepared = false;
  e->cell_factor = cell_factor;
  e->visit_sorted = visit_sorted ? 1 : 0;
  ens_drop_graphs(e);
  return ABL_OK;
}

int abl_ensemble_set_tiling(abl_ensemble *e, int entries) {
  if (!e || entries < 0 || entries > 4096 || entries % 256) return ABL_E_INVALID;
  if (entries != e->base.block_cap) e->prepared = false;  // views carry it
  e->base.block_cap = entries;
  ens_drop_graphs(e);
  return ABL_OK;
}

int abl_ensemble_set_persistent(abl_ensemble *e, int enable) {
  if (!e) return ABL_E_INVALID;
  if (enable && !e->base.model->launch_ens_persist) return ABL_E_UNSUPPORTED;
  e->persistent = enable != 0;
  return ABL_OK;
}

int abl_ensemble_persistent_blocks(abl_ensemble *e, int *blocks) {
  if (!e || !blocks) return ABL_E_INVALID;
  *blocks = e->persist_grid;
  return ABL_OK;
}

int abl_ensemble_phase_times(abl_ensemble *e, double *seconds, int cap, int *count) {
  if (!e || !count || cap < 0 || (cap > 0 && !seconds)) return ABL_E_INVALID;
  *count = 0;
  if (!e->d_stamps) return ABL_OK;
  unsigned long long st[kPersistStamps];
  ABL_CUDA_TRY(cudaMemcpy(st, e->d_stamps, sizeof st, cudaMemcpyDeviceToHost));
  int n = 0;
  while (n < kPersistStamps && st[n] != 0) n++;
  for (int k = 0; k + 1 < n && k < cap; k++) seconds[k] = (double) (st[k + 1] - st[k]) * 1e-9;
  *count = std::max(0, std::min(n - 1, cap));
  return ABL_OK;
}

int abl_diag_ensemble_barrier(void *ensemble, double limit_seconds, int extra_arrivals) {
  abl_ensemble *e = (abl_ensemble *) ensemble;
  if (!e || limit_seconds < 0.0 || limit_seconds > 60.0 || extra_arrivals < 0 ||
      extra_arrivals > 1)
    return ABL_E_INVALID;
  e->barrier_limit_ns = limit_seconds > 0.0 ? (unsigned long long) (limit_seconds * 1e9)
                                            : 4000000000ull;
  e->barrier_extra = (unsigned int) extra_arrivals;
  return ABL_OK;
}

int abl_ensemble_get_tuning(abl_ensemble *e, int *block, double *cell_factor, int *visit_sorted,
                            int *tiling_entries) {
  if (!e) return ABL_E_INVALID;
  if (block) *block = e->block;
  if (cell_factor) *cell_factor = e->cell_factor;
  if (visit_sorted) *visit_sorted = e->visit_sorted;
  if (tiling_entries) *tiling_entries = e->base.block_cap;
  return ABL_OK;
}

// Tries every combination of block size, cell size factor, visiting order and
// (with cell-order visits) block tiling for `trial_timesteps` timesteps
// (after one warm-up timestep) and keeps the fastest.  The state and timestep counter are restored after each trial, so
// tuning does not advance the simulation; every candidate computes identical
// results.
int abl_ensemble_autotune(abl_ensemble *e, int trial_timesteps, int *block, double *cell_factor,
                          int *visit_sorted) {
  if (!e || trial_timesteps <= 0) return ABL_E_INVALID;
  ABL_TRY(ens_ready(e));
  abl_ctx *ctx = &e->base;
  // Snapshot of the current state.
  std::vector<std::vector<void *>> snap(e->types.size());
  std::vector<int> cur(e->types.size());
  for (size_t ti = 0; ti < e->types.size(); ti++) {
    EnsType &t = e->types[ti];
    cur[ti] = t.cur;
    for (int k = 0; k < t.d->num_members; k++) {
      void *p = nullptr;
      size_t bytes = member_bytes(t.d->members[k]) * std::max<long>(t.n, 1);
      ABL_TRY(dev_alloc(ctx, &p, bytes));
      ABL_CUDA_TRY(cudaMemcpyAsync(p, t.cols[t.cur][k], bytes, cudaMemcpyDeviceToDevice,
                                   ctx->stream));
      snap[ti].push_back(p);
    }
  }
  auto restore = [&]() -> int {
    for (size_t ti = 0; ti < e->types.size(); ti++) {
      EnsType &t = e->types[ti];
      t.cur = cur[ti];
      t.dirty = true;
      for (int k = 0; k < t.d->num_members; k++) {
        size_t bytes = member_bytes(t.d->members[k]) * std::max<long>(t.n, 1);
        ABL_CUDA_TRY(cudaMemcpyAsync(t.cols[t.cur][k], snap[ti][k], bytes,
                                     cudaMemcpyDeviceToDevice, ctx->stream));
      }
    }
    return ABL_OK;
  };
  long ts0 = e->timestep;
  const int blocks[] = {64, 128};
  const double factors[] = {1.0, 1.5, 2.0};
  const int visits[] = {1, 0};
  const int tilings[] = {2048, 1024, 4096, 0};
  double best = 1e30;
  int bb = e->block, bv = e->visit_sorted, bt = e->base.block_cap;
  double bf = e->cell_factor;
  for (int b : blocks) {
    for (double f : factors) {
      for (int v : visits) {
        for (int tl : tilings) {
          if (!v && tl != tilings[0]) continue;  // tiling needs cell-order visits
          ABL_TRY(abl_ensemble_set_tuning(e, b, f, v));
          ABL_TRY(abl_ensemble_set_tiling(e, tl));
          ABL_TRY(ens_ready(e));
          ABL_TRY(restore());
          e->timestep = ts0;
          ABL_TRY(abl_ensemble_run(e, 1));
          ABL_TRY(abl_ensemble_run(e, trial_timesteps));
          double t = ctx->last_exec;
          if (t < best) {
            best = t;
            bb = b;
            bf = f;
            bv = v;
            bt = tl;
          }
        }
      }
    }
  }
  ABL_TRY(abl_ensemble_set_tuning(e, bb, bf, bv));
  ABL_TRY(abl_ensemble_set_tiling(e, bt));
  ABL_TRY(ens_ready(e));
  ABL_TRY(restore());
  ABL_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  for (auto &v : snap)
    for (void *p : v) dev_free(ctx, p);
  e->timestep = ts0;
  if (block) *block = bb;
  if (cell_factor) *cell_factor = bf;
  if (visit_sorted) *visit_sorted = bv;
  return ABL_OK;
}

int abl_ensemble_last_exec_time(abl_ensemble *e, double *seconds) {
  if (!e || !seconds) return ABL_E_INVALID;
  *seconds = e->base.last_exec;
  return ABL_OK;
}

int abl_ensemble_last_launch_count(abl_ensemble *e, long *launches) {
  if (!e || !launches) return ABL_E_INVALID;
  *launches = e->base.last_launches;
  return ABL_OK;
}

int abl_ensemble_destroy(abl_ensemble *e) {
  if (!e) return ABL_E_INVALID;
  abl_ctx *ctx = &e->base;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  ens_drop_graphs(e);
  for (void *p : ctx->allocations) cudaFreeAsync(p, ctx->stream);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  ctx->allocations.clear();
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  ctx->stream = nullptr;
  delete e;
  return ABL_OK;
}

}  // extern "C"
