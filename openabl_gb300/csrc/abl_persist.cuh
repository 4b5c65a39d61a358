// Persistent ensemble kernel: every phase of every timestep of an ensemble
// run in ONE cooperative launch.
//
// The graph-replayed ensemble timestep is a sequence of kernels over the
// segmented grid of all replicas (assign, scan, scatter, sort, gather, lists,
// step).  Here one grid of co-resident blocks (a cooperative launch, so every
// block is resident and a grid-wide barrier cannot wait on a block that never
// started) runs those phases back to back, separated by grid-wide barriers,
// for all timesteps of the run.  Work is the same per item: the phases call
// the items of abl_bin.cuh and the generated step bodies, so every replica
// computes the bits a separate context computes.
//
// Phases of the binning of one agent type (2D row lists; `levels` list
// levels in all):
//   assign -> scan A -> scan C -> scatter + list counts + count reset
//   -> sort + list scan A -> gather + list scan C -> merge (level 0)
//   [-> list scan A -> list scan C -> merge (next level) ...]
// then one phase per step function.  Independent work shares a phase:
// the list counts need only the cell starts, so they run beside the scatter.
//
// Waits.  The only waits are the grid barriers.  Each gives up after a time
// limit (globaltimer), records ABL_E_TIMEOUT in the sync word and makes the
// block return; a block that sees another block's error returns too.  So a
// launch always ends, and the host reads the error word afterwards.
//
// Memory.  Grids are rewritten between phases of one launch, so this header
// is compiled with ABL_PERSIST, which makes ABL_LDG a plain (coherent) load:
// the read-only data path may return lines cached before the rewrite.
#pragma once

#include "abl_bin.cuh"

// Resident blocks per SM the persistent kernel's register allocation must
// allow (its step phase is the step kernel's body).
// Five blocks of 128 threads leave 96 registers a thread; with six (80) the
// step body spills (measured on 200 timesteps of the 256-replica FP32
// boids2d ensemble: 1.67 s with five blocks, 1.82 s with six).
#ifndef ABL_PERSIST_MIN_BLOCKS
#define ABL_PERSIST_MIN_BLOCKS 5
#endif

namespace abl {

enum { kPersistBin = 0, kPersistStep = 1 };
// Items a thread of the persistent kernel takes at a time in the gathering
// phases, loads first: the binning phases run at the step phase's
// occupancy, so each thread keeps more loads in flight than in the
// per-phase kernels.  (Two: four spill more registers in the step phase;
// 200 timesteps of the 256-replica FP32 boids2d ensemble took 1.65 s with
// two, 1.67 s with four.)
#ifndef ABL_PERSIST_ILP
#define ABL_PERSIST_ILP 2
#endif
constexpr int kPersistILP = ABL_PERSIST_ILP;
constexpr int kPersistMaxOps = 16;    // ops (binnings + step functions) per timestep
constexpr int kPersistMaxLevels = 3;  // list levels (3D ordered lists)

// Binning of one agent type over all replicas.
struct persist_bin {
  int dim, pos_double, levels, Rmax;
  long n, ncells;
  const void *pos;
  const int *replica_of;
  const ablbin::EnsGrid *grids;
  const int *cell_replica;
  int *cell_of, *cell_count, *local_rank, *order, *cell_start;
  float *posf;
  float *amax;      // read by the step functions' views
  float *amax_acc;  // assign phase accumulator, copied to amax and reset
  int *scan_incl, *scan_sums;  // ncells, one per chunk
  ablbin::GatherArgs gather;
  // list level a: counts -> dst_off[a] (ncells + 1), then elements
  // dst_elem[a] or, for the last level of ordered lists, slots dst_slot[a]
  int *cnt;
  int *dst_off[kPersistMaxLevels];
  int4 *dst_elem[kPersistMaxLevels];
  int *dst_slot[kPersistMaxLevels];
};

struct persist_op {
  int kind;  // kPersistBin / kPersistStep
  persist_bin bin;
  abl_ens_launch step;
};

struct persist_timestep {
  int nops;
  persist_op ops[kPersistMaxOps];
};

struct persist_sync {
  unsigned int count;  // blocks arrived at the current barrier
  unsigned int gen;    // barrier generation
  int error;           // ABL_E_TIMEOUT once a wait gave up
  int pad;
  // Virtual blocks of the step phases handed out so far (one counter for
  // the whole run; each phase's share starts where the last one's ended).
  unsigned long long work;
};

// A run: timesteps [0, timesteps) use ts[0] for the first one when
// `first_special`, and then ts[a], ts[b] alternately (the runtime's double
// buffers flip every timestep, so the pointer sets repeat with period two).
struct persist_prog {
  long timesteps;
  long base_timestep;  // timestep number of the first one (random() keys on it)
  int first_special;
  persist_timestep ts[3];
  persist_sync *sync;
  unsigned long long limit_ns;  // longest wait at one barrier
  unsigned int extra_arrivals;  // arrivals a barrier waits for beyond the grid's blocks
  int scan_chunk;               // ints per scan chunk
  // Phase timestamps (globaltimer ns, NULL: none): block 0 records when
  // each barrier completed, the first `stamp_cap` of them.
  unsigned long long *stamps;
  int stamp_cap;
};

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int *p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(unsigned int *p, unsigned int v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid-wide barrier of `expected` arrivals.  Every thread of every block
// calls it; returns false (uniformly over the block) when the wait gave up
// or another block's did.
__device__ inline bool grid_barrier(persist_sync *s, unsigned int expected,
                                    unsigned long long limit_ns) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    // The generation cannot change before this block has arrived.
    const unsigned int g = ld_acquire(&s->gen);
    __threadfence();
    const unsigned int arrived = atomicAdd(&s->count, 1u) + 1u;
    int good = 1;
    if (arrived == expected) {
      // Every other block's fence and arrival precede this arrival in the
      // count's order: the fence acquires their writes, and the release of
      // the new generation passes them on to the blocks that wait for it.
      __threadfence();
      atomicExch(&s->count, 0u);
      st_release(&s->gen, g + 1u);
    } else {
      const unsigned long long t0 = global_ns();
      while (ld_acquire(&s->gen) == g) {
        if (ld_acquire(&s->error) != 0) {
          good = 0;
          break;
        }
        if (global_ns() - t0 > limit_ns) {
          atomicCAS(&s->error, 0, ABL_E_TIMEOUT);
          good = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    ok = good && ld_acquire(&s->error) == 0;
  }
  __syncthreads();
  return ok != 0;
}

// Block-wide exclusive scan of one int per thread; returns the thread's
// prefix and sets *total.  Every thread calls it.
__device__ inline int block_exclusive_scan(int v, int *total) {
  __shared__ int warp_sum[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sum[w] = x;
  __syncthreads();
  if (w == 0) {
    int s = lane < nw ? warp_sum[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < nw) warp_sum[lane] = s;
  }
  __syncthreads();
  const int before = w > 0 ? warp_sum[w - 1] : 0;
  *total = warp_sum[nw - 1];
  __syncthreads();  // warp_sum is reused by the next call
  return before + x - v;
}

// Chunks [c0, c1) of this block when `nchunks` are split into contiguous
// ranges over the grid.
__device__ __forceinline__ void block_chunks(long nchunks, long &c0, long &c1) {
  const long per = (nchunks + gridDim.x - 1) / gridDim.x;
  c0 = (long) blockIdx.x * per;
  c1 = c0 + per < nchunks ? c0 + per : nchunks;
}

// Scan phase A: inclusive scan of each chunk of `in` (m ints) into incl,
// the chunk's total into sums.
__device__ inline void scan_phase_a(const int *in, long m, int chunk, int *incl, int *sums) {
  const long nchunks = (m + chunk - 1) / chunk;
  long c0, c1;
  block_chunks(nchunks, c0, c1);
  // Thread t takes the `per` consecutive elements from t * per of a chunk.
  const int per = (chunk + blockDim.x - 1) / blockDim.x;
  const int first = threadIdx.x * per;
  const int mine = first >= chunk ? 0 : (first + per <= chunk ? per : chunk - first);
  for (long c = c0; c < c1; c++) {
    const long base = c * chunk + first;
    int run = 0;
    for (int k = 0; k < mine; k++) run += base + k < m ? in[base + k] : 0;
    int total;
    int prefix = block_exclusive_scan(run, &total);
    for (int k = 0; k < mine; k++) {
      if (base + k < m) {
        prefix += in[base + k];
        incl[base + k] = prefix;
      }
    }
    if (threadIdx.x == 0) sums[c] = total;
  }
}

// Scan phase C: out[0] = 0, out[j + 1] = incl[j] + the totals of the chunks
// before j's.  A block's chunks are contiguous, so it adds up the totals
// before its first chunk once and carries them on.
__device__ inline void scan_phase_c(const int *incl, const int *sums, long m, int chunk,
                                    int *out) {
  const long nchunks = (m + chunk - 1) / chunk;
  long c0, c1;
  block_chunks(nchunks, c0, c1);
  if (c0 >= c1) {
    if (m == 0 && blockIdx.x == 0 && threadIdx.x == 0) out[0] = 0;
    return;
  }
  int part = 0;
  for (long c = threadIdx.x; c < c0; c += blockDim.x) part += sums[c];
  int offset;
  block_exclusive_scan(part, &offset);
  for (long c = c0; c < c1; c++) {
    for (long j = c * chunk + threadIdx.x; j < (c + 1) * chunk && j < m; j += blockDim.x)
      out[j + 1] = incl[j] + offset;
    offset += sums[c];
  }
  if (c0 == 0 && threadIdx.x == 0) out[0] = 0;
}

__device__ __forceinline__ long grid_thread() {
  return (long) blockIdx.x * blockDim.x + threadIdx.x;
}
__device__ __forceinline__ long grid_threads() { return (long) gridDim.x * blockDim.x; }

static_assert(sizeof(abl_ens_launch) % 8 == 0 && alignof(abl_ens_launch) == 8 &&
                  sizeof(persist_bin) % 8 == 0 && alignof(persist_bin) == 8,
              "op arguments are copied as 8-byte words");

// Block-wide copy of `bytes` (a multiple of 8) from global to shared memory.
__device__ __forceinline__ void copy_words(void *dst, const void *src, size_t bytes) {
  for (int w = threadIdx.x; w < (int) (bytes / 8); w += blockDim.x)
    ((unsigned long long *) dst)[w] = ((const unsigned long long *) src)[w];
}

// State of one block's walk through the run.  Its position (timestep, op,
// virtual block, the phase timestamps taken) lives in shared memory and is
// written by thread 0 between barriers, so that across a step body nothing
// is live but kernel parameters and shared memory, and the body keeps the
// registers to itself.
struct persist_cursor {
  long it;                       // timestep of the run
  long ts;                       // its number (random() keys on it)
  long nvb, vb;                  // step phase: virtual blocks, the one to run
  unsigned long long work_base;  // the counter's value where this phase's share starts
  int o;                         // op of the timestep
  int nstamps;                   // phase timestamps taken (block 0)
};

struct persist_walk {
  const persist_prog *P;
  int *error;
  int *stage;
  persist_cursor *C;

  // Grid barrier; block 0 then records when the phase ended.
  __device__ bool sync() {
    if (!grid_barrier(P->sync, gridDim.x + P->extra_arrivals, P->limit_ns)) return false;
    if (P->stamps && blockIdx.x == 0 && threadIdx.x == 0 && C->nstamps < P->stamp_cap)
      P->stamps[C->nstamps++] = global_ns();
    return true;
  }
};

template <typename Real, int DIM>
__device__ float persist_assign(const persist_bin &B, int *error) {
  float m = 0.0f;
  const Real *pos = (const Real *) B.pos;
  for (long i = grid_thread(); i < B.n; i += grid_threads())
    m = fmaxf(m, ablbin::ens_bin_assign_item<Real, DIM>(i, pos, B.replica_of, B.grids,
                                                        B.cell_of, B.cell_count, B.local_rank,
                                                        error));
  return m;
}

// Slot-ordered copies (as gather_item), kPersistILP slots at a time.
template <typename Real, int DIM>
__device__ void persist_gather(const persist_bin &B) {
  constexpr int U = kPersistILP;
  const Real *pos = (const Real *) B.pos;
  const ablbin::GatherArgs &g = B.gather;
  const long T = grid_threads();
  for (long s0 = grid_thread(); s0 < B.n; s0 += U * T) {
    long idx[U];
#pragma unroll
    for (int u = 0; u < U; u++) idx[u] = s0 + u * T < B.n ? B.order[s0 + u * T] : -1;
    if (B.posf) {
      Real p[U][DIM];
#pragma unroll
      for (int u = 0; u < U; u++)
#pragma unroll
        for (int d = 0; d < DIM; d++) p[u][d] = idx[u] >= 0 ? pos[DIM * idx[u] + d] : Real(0);
#pragma unroll
      for (int u = 0; u < U; u++)
        if (idx[u] >= 0)
#pragma unroll
          for (int d = 0; d < DIM; d++) B.posf[DIM * (s0 + u * T) + d] = (float) p[u][d];
    }
    for (int k = 0; k < g.nmem; k++) {
      const int b = g.bytes[k];
      if ((b & 7) == 0) {
        for (int w = 0; w < b / 8; w++) {
          uint64_t v[U];
#pragma unroll
          for (int u = 0; u < U; u++)
            if (idx[u] >= 0) v[u] = ((const uint64_t *) g.src[k])[(b / 8) * idx[u] + w];
#pragma unroll
          for (int u = 0; u < U; u++)
            if (idx[u] >= 0) ((uint64_t *) g.dst[k])[(b / 8) * (s0 + u * T) + w] = v[u];
        }
      } else if ((b & 3) == 0) {
        for (int w = 0; w < b / 4; w++) {
          uint32_t v[U];
#pragma unroll
          for (int u = 0; u < U; u++)
            if (idx[u] >= 0) v[u] = ((const uint32_t *) g.src[k])[(b / 4) * idx[u] + w];
#pragma unroll
          for (int u = 0; u < U; u++)
            if (idx[u] >= 0) ((uint32_t *) g.dst[k])[(b / 4) * (s0 + u * T) + w] = v[u];
        }
      } else {
        for (int w = 0; w < b; w++) {
          uint8_t v[U];
#pragma unroll
          for (int u = 0; u < U; u++)
            if (idx[u] >= 0) v[u] = ((const uint8_t *) g.src[k])[b * idx[u] + w];
#pragma unroll
          for (int u = 0; u < U; u++)
            if (idx[u] >= 0) ((uint8_t *) g.dst[k])[b * (s0 + u * T) + w] = v[u];
        }
      }
    }
  }
}

// Counting-sort placement (as bin_scatter_item), kPersistILP agents at a
// time; the cell counts, consumed by the scan, are reset for the next
// binning in the same pass.
__device__ inline void persist_scatter(const persist_bin &B) {
  constexpr int U = kPersistILP;
  const long T = grid_threads();
  for (long i0 = grid_thread(); i0 < B.n; i0 += U * T) {
    int cell[U], rank[U], start[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const long i = i0 + u * T;
      cell[u] = i < B.n ? B.cell_of[i] : 0;
      rank[u] = i < B.n ? B.local_rank[i] : 0;
    }
#pragma unroll
    for (int u = 0; u < U; u++) start[u] = i0 + u * T < B.n ? B.cell_start[cell[u]] : 0;
#pragma unroll
    for (int u = 0; u < U; u++)
      if (i0 + u * T < B.n) B.order[start[u] + rank[u]] = (int) (i0 + u * T);
  }
  for (long c = grid_thread(); c < B.ncells; c += T) B.cell_count[c] = 0;
}

// DIM 2 or 3 with Real the position's scalar: the model's one kind of
// binned position, fixed when the kernel is generated.  DIM 0: chosen per
// binning from the program.
template <typename Real, int DIM>
__device__ __forceinline__ float assign_any(const persist_bin &B, int *error) {
  if constexpr (DIM != 0) {
    return persist_assign<Real, DIM>(B, error);
  } else {
    if (B.pos_double) return B.dim == 2 ? persist_assign<double, 2>(B, error)
                                        : persist_assign<double, 3>(B, error);
    return B.dim == 2 ? persist_assign<float, 2>(B, error) : persist_assign<float, 3>(B, error);
  }
}

template <typename Real, int DIM>
__device__ __forceinline__ void gather_any(const persist_bin &B) {
  if constexpr (DIM != 0) {
    persist_gather<Real, DIM>(B);
  } else {
    if (B.pos_double) {
      if (B.dim == 2) persist_gather<double, 2>(B);
      else persist_gather<double, 3>(B);
    } else {
      if (B.dim == 2) persist_gather<float, 2>(B);
      else persist_gather<float, 3>(B);
    }
  }
}

template <int AXIS>
__device__ void persist_count(const persist_bin &B, const ablbin::EnsGeom &geo, const int *src_off) {
  for (long c = grid_thread(); c < B.ncells; c += grid_threads())
    ablbin::sep_count_item<ablbin::EnsGeom, AXIS>(c, geo, src_off, B.cnt);
}

// List level a (R = 1 cells: one thread per cell at level 0, one warp per
// cell above; R > 1 cells: one warp per cell).  `stage`: kSepStage ints of
// shared memory per warp.
template <int AXIS>
__device__ void persist_merge(const persist_bin &B, const ablbin::EnsGeom &geo,
                              const ablbin::SepSrc &S, int *stage) {
  const int lane = threadIdx.x & 31;
  const long warp = grid_thread() >> 5, warps = grid_threads() >> 5;
  if constexpr (AXIS == 0) {
    for (long t = grid_thread(); t < B.ncells; t += grid_threads())
      ablbin::sep_merge_item<ablbin::EnsGeom, 0, true>(t, geo, S, B.dst_off[0], B.dst_elem[0],
                                                      B.dst_slot[0]);
  } else {
    int *my = stage + (threadIdx.x >> 5) * ablbin::kSepStage;
    for (long t = warp; t < B.ncells; t += warps)
      ablbin::sep_merge_warp_item<ablbin::EnsGeom, AXIS, false>(t, lane, geo, S, B.dst_off[AXIS],
                                                               B.dst_elem[AXIS],
                                                               B.dst_slot[AXIS], my);
  }
  if (B.Rmax > 1) {
    for (long t = warp; t < B.ncells; t += warps)
      ablbin::sep_merge_large_item<ablbin::EnsGeom, AXIS>(t, lane, geo, S, B.dst_off[AXIS],
                                                         B.dst_elem[AXIS], B.dst_slot[AXIS]);
  }
}

// Counts of list level a (sources: the cells' runs at level 0, else level
// a - 1's lists).  Axes beyond the positions' dimension never occur.
template <int DIM>
__device__ inline void persist_count_dispatch(const persist_bin &B, const ablbin::EnsGeom &geo,
                                              int a) {
  if (a == 0) persist_count<0>(B, geo, B.cell_start);
  else if (a == 1) persist_count<1>(B, geo, B.dst_off[0]);
  else if (DIM != 2) persist_count<2>(B, geo, B.dst_off[1]);
}

template <int DIM>
__device__ inline void persist_merge_dispatch(const persist_bin &B, const ablbin::EnsGeom &geo,
                                              int a, int *stage) {
  if (a == 0) {
    persist_merge<0>(B, geo, ablbin::SepSrc{B.cell_start, B.order, B.posf, B.dim, nullptr},
                     stage);
    return;
  }
  const ablbin::SepSrc S{B.dst_off[a - 1], nullptr, nullptr, B.dim, B.dst_elem[a - 1]};
  if (a == 1) persist_merge<1>(B, geo, S, stage);
  else if (DIM != 2) persist_merge<2>(B, geo, S, stage);
}

// The binning of one type: returns false when a barrier gave up.
template <typename Real, int DIM>
__device__ inline bool persist_binning(persist_walk &W, const persist_bin &B) {
  const int chunk = W.P->scan_chunk;
  // assign
  const float m = assign_any<Real, DIM>(B, W.error);
  ablbin::fold_amax(m, B.amax_acc);
  if (!W.sync()) return false;
  scan_phase_a(B.cell_count, B.ncells, chunk, B.scan_incl, B.scan_sums);
  if (!W.sync()) return false;
  scan_phase_c(B.scan_incl, B.scan_sums, B.ncells, chunk, B.cell_start);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *B.amax = *B.amax_acc;
    *B.amax_acc = 0.0f;
  }
  if (!W.sync()) return false;
  // scatter; the counts of list level 0 need only the cell starts; the cell
  // counts are consumed, so they are reset for the next binning here
  const ablbin::EnsGeom geo{B.cell_replica, B.grids};
  persist_scatter(B);
  if (B.levels > 0) persist_count_dispatch<DIM>(B, geo, 0);
  if (!W.sync()) return false;
  for (long c = grid_thread(); c < B.ncells; c += grid_threads())
    ablbin::cell_sort_item(c, B.cell_start, B.order);
  if (B.levels > 0) scan_phase_a(B.cnt, B.ncells, chunk, B.scan_incl, B.scan_sums);
  if (!W.sync()) return false;
  gather_any<Real, DIM>(B);
  if (B.levels > 0) scan_phase_c(B.scan_incl, B.scan_sums, B.ncells, chunk, B.dst_off[0]);
  if (!W.sync()) return false;
  for (int a = 0; a < B.levels; a++) {
    persist_merge_dispatch<DIM>(B, geo, a, W.stage);
    if (a + 1 < B.levels) persist_count_dispatch<DIM>(B, geo, a + 1);
    if (!W.sync()) return false;
    if (a + 1 < B.levels) {
      scan_phase_a(B.cnt, B.ncells, chunk, B.scan_incl, B.scan_sums);
      if (!W.sync()) return false;
      scan_phase_c(B.scan_incl, B.scan_sums, B.ncells, chunk, B.dst_off[a + 1]);
      if (!W.sync()) return false;
    }
  }
  return true;
}

// The whole run.  `body(L, vb, ts)` runs the step function L.step_index
// for virtual block vb (the agents vb * blockDim.x ...) at timestep ts; it
// is the generated ensemble step body.  `error` is the context's error word
// (non-finite positions).  Real and DIM: see assign_any.
template <typename Real, int DIM, typename Body>
__device__ void persist_run(const persist_prog *Pp, int *error, Body &&body) {
  extern __shared__ int abl_presort_dyn[];
  // The step's launch block and the binning's arguments, copied to shared
  // memory for each op: read at shared-memory latency.
  __shared__ abl_ens_launch Ls;
  __shared__ persist_bin Bs;
  __shared__ persist_cursor C;
  // List staging shares the step's dynamic shared memory.
  persist_walk W{Pp, error, abl_presort_dyn, &C};
  if (threadIdx.x == 0) {
    C.it = 0;
    C.o = 0;
    C.work_base = 0;
    C.nstamps = 0;
  }
  // Cell counts and coordinate maxima start at zero.
  for (int k = 0; k < 3; k++) {
    const persist_timestep &T = Pp->ts[k];
    for (int o = 0; o < T.nops; o++) {
      const persist_op &op = T.ops[o];
      if (op.kind != kPersistBin) continue;
      for (long c = grid_thread(); c < op.bin.ncells; c += grid_threads()) op.bin.cell_count[c] = 0;
      if (grid_thread() == 0) *op.bin.amax_acc = 0.0f;
    }
  }
  if (!W.sync()) return;
  for (;;) {
    const long it = C.it;
    if (it >= Pp->timesteps) break;
    const int k = Pp->first_special ? (it == 0 ? 0 : 1 + (int) ((it - 1) & 1)) : (int) (it & 1);
    const persist_timestep &T = Pp->ts[k];
    const persist_op &op = T.ops[C.o];
    if (op.kind == kPersistBin) {
      copy_words(&Bs, &op.bin, sizeof(persist_bin));
      __syncthreads();
      if (!persist_binning<Real, DIM>(W, Bs)) return;
    } else {
      // Step phases hand out virtual blocks dynamically, as the hardware
      // hands out a kernel's blocks (agents' neighbour counts vary, so fixed
      // shares would finish unevenly).  A block claims its next virtual
      // block while it runs the current one.  Every block makes one claim
      // past the end, so the next phase's share starts nvb + gridDim.x on.
      copy_words(&Ls, &op.step, sizeof(abl_ens_launch));
      if (threadIdx.x == 0) {
        C.ts = Pp->base_timestep + it;
        C.nvb = (op.step.n + blockDim.x - 1) / blockDim.x;
        C.vb = (long) (atomicAdd(&Pp->sync->work, 1ull) - C.work_base);
      }
      __syncthreads();
      while (C.vb < C.nvb) {  // uniform over the block
        unsigned long long next = 0;
        if (threadIdx.x == 0) next = atomicAdd(&Pp->sync->work, 1ull);
        body(Ls, C.vb, C.ts);
        __syncthreads();  // shared memory is reused by the next virtual block
        if (threadIdx.x == 0) C.vb = (long) (next - C.work_base);
        __syncthreads();
      }
      if (threadIdx.x == 0) C.work_base += (unsigned long long) C.nvb + gridDim.x;
      if (!W.sync()) return;
    }
    if (threadIdx.x == 0 && ++C.o >= T.nops) {
      C.o = 0;
      C.it++;
    }
    __syncthreads();
  }
}

// Host side of abl_persist_launch_fn for a model's persistent kernel: the
// grid is at most every block that can be resident at once (a cooperative
// launch refuses more), so a grid barrier never waits on a block that has
// not started; *grid > 0 on entry caps it (small ensembles: fewer blocks to
// synchronise at every barrier).
inline int persist_launch(const void *kernel, const void *prog, int *err, int block, size_t smem,
                          int *grid, cudaStream_t stream) {
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem)
          != cudaSuccess)
    return ABL_E_CUDA;
  int per_sm = 0, dev = 0, sms = 0, coop = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem) != cudaSuccess)
    return ABL_E_CUDA;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess)
    return ABL_E_CUDA;
  if (!coop || per_sm < 1) return ABL_E_UNSUPPORTED;
  int g = per_sm * sms;
  if (grid && *grid > 0 && *grid < g) g = *grid;
  if (grid) *grid = g;
  if (!prog) return ABL_OK;
  void *args[2] = {(void *) &prog, (void *) &err};
  return cudaLaunchCooperativeKernel(kernel, dim3(g), dim3(block), args, smem, stream)
                 == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}

}  // namespace abl
