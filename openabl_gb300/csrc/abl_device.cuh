// Device-side helpers shared by the runtime and generated step kernels.
//
// Neighbour iteration.  The reference `near` loop visits every agent of the
// neighbour type in ascending index and skips those with
// dist(nx.pos, in.pos) > radius (src/backend/CPrinter.cpp:148-173), where
// dist is sqrtf of the double sum of squares (asset/c/libabl.h:156-168).
// Here the neighbour type is binned into a uniform grid whose cells are at
// least as wide as any near radius; an agent's candidates are the agents in
// the cells within `range` of its own cell.
//
//  * Ordered mode (bodies whose result depends on the visiting order, e.g.
//    floating-point accumulation): the runtime builds, per cell, the list of
//    candidate slots in ascending agent id, so the body sees exactly the
//    reference's sequence of in-radius neighbours.
//  * Unordered mode (bodies that only do integer accumulation): candidates
//    are walked cell row by cell row without sorting.
//  * Presorted mode (ordered bodies of a step's single near loop around the
//    step's own agent): before any step body runs, each thread of a block
//    collects the in-radius neighbours of one of the block's agents and keeps
//    them in shared memory sorted by agent id (at most a fixed number at a
//    time; more are fetched again past the last one consumed).  Optionally
//    the block then hands its agents to its threads in ascending order of
//    neighbour count, so the lanes of a warp run loop bodies of nearly equal
//    length.  No global neighbourhood lists are built.
//
// The radius test is decided without FP64 arithmetic for almost every
// candidate: the squared distance is computed in FP32 from float copies of
// the positions and compared against [r^2 (1 - eps), r^2 (1 + eps)], where
// eps bounds the error of that FP32 estimate relative to the reference's
// double computation (given the largest coordinate magnitude A of the agents
// involved).  Candidates inside that band fall back to the generated exact
// test, which evaluates the reference expression itself.  Passing slots are
// buffered per thread in ascending order and the loop body then runs over the
// buffer, so the FP64 body work is not fragmented by the filter's branches.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <type_traits>

#include "abl_model.h"

// Loads of data that no kernel writes while the reading kernel runs go
// through the read-only (non-coherent) data path.  The persistent ensemble
// kernel rewrites its grids between phases of one launch, where that path
// could return lines cached before the rewrite, so its translation units are
// compiled with ABL_PERSIST and use plain (coherent) loads.  ABL_PLAIN_LOADS
// selects plain loads for every kernel (a build option for comparing the
// two paths).
#if defined(ABL_PERSIST) || defined(ABL_PLAIN_LOADS)
#define ABL_LDG(p) (*(p))
#else
#define ABL_LDG(p) __ldg(p)
#endif

#ifndef ABL_NEAR_CHUNK
#define ABL_NEAR_CHUNK 32
#endif
// Step kernels run with at most this many threads per block; each thread
// owns one column of the block's shared chunk buffer.
#ifndef ABL_STEP_BLOCK
#define ABL_STEP_BLOCK 128
#endif
// Resident step-kernel blocks per SM the register allocation must allow.
// Six blocks of 128 threads cap a step kernel at 80 registers: the FP64
// boids2d body fits without spilling, and the extra resident warps hide the
// latency of the neighbour gathering (measured: 1M boids2d step kernel
// 0.74 -> 0.67 ms against no cap; eight blocks gain nothing more and spill).
// Neighbours held per agent in a presorted kernel's shared-memory column
// (agents with more take further chunks).
#ifndef ABL_LIST_CAP
#define ABL_LIST_CAP 32
#endif
#ifndef ABL_STEP_MIN_BLOCKS
#define ABL_STEP_MIN_BLOCKS 6
#endif

namespace abl {

// FP64 additions on this GPU issue faster as fused multiply-adds than as
// adds (measured: abl_diag_fp64_add_as_fma_rate against abl_diag_fp64_rates).
// fma(a, 1, b) rounds a * 1 + b = a + b once, so it is the same correctly
// rounded sum (signed zeros included); a - b is fma(b, -1, a).  The 1.0 lives
// in constant memory so that the compiler cannot fold the fma back into an
// add.
static __constant__ double fp64_one = 1.0;
__device__ __forceinline__ double dadd(double a, double b) { return __fma_rn(a, fp64_one, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __fma_rn(b, -fp64_one, a); }

// Cell coordinate of x along one axis; out-of-range positions are clamped
// into the border cells (monotone, so neighbours within one cell width stay
// within one cell index).
__host__ __device__ inline int cell_coord(double x, double lo, double inv_cell, int n) {
  double f = floor((x - lo) * inv_cell);
  if (!(f > 0.0)) return 0;
  if (f >= (double) (n - 1)) return n - 1;
  return (int) f;
}

// The same in FP32 arithmetic, for grids whose size and offset keep its
// rounding error far inside the cells' 2^-10 margin (the runtime decides,
// bin_in_fp32): monotone in x, clamped into the border cells.
__host__ __device__ inline int cell_coord_f32(float x, float lo, float inv_cell, int n) {
#ifdef __CUDA_ARCH__
  const float f = floorf(__fmul_rn(__fsub_rn(x, lo), inv_cell));
#else
  const float f = floorf((x - lo) * inv_cell);
#endif
  if (!(f > 0.0f)) return 0;
  if (f >= (float) (n - 1)) return n - 1;
  return (int) f;
}

struct band {
  float lo, hi;
};

// Prefilter band for radius r.  u = 2^-24.  For a pair whose reference test
// is near the threshold, |dx| <= s ~ 1.1 r; float rounding of the two
// positions (|x| <= A) and of the FP32 subtraction perturbs dx by at most
// E = 2uA + u s per axis, hence d2 by dim * E (2 s + E); the FP32 squares and
// sum and the reference's own rounding chain (double or float arithmetic, the
// float rounding of d2 and sqrtf) add a few u relative.  eps doubles that sum.
// When eps is not small (huge coordinates, zero or negative radius, non-finite
// values) every candidate takes the exact test.
__device__ inline band make_band(float r, float amax, int dim) {
  band b;
  b.lo = -1.0f;
  b.hi = __int_as_float(0x7f800000);  // +inf: nothing is decided by the filter
  if (!(r > 0.0f) || !(r < 1e15f) || !(amax >= 0.0f) || !(amax < 1e30f)) return b;
  const float u = 5.9604645e-8f;
  float s = 1.1f * r;
  float E = (2.0f * u * amax + u * s) * 1.01f;
  s += E;
  float mp = (float) dim * E * (2.0f * s + E);
  float r2 = r * r;
  float eps = 2.0f * (mp / r2 + 16.0f * u) + 4.0e-7f;
  if (!(eps < 0.1f)) return b;
  b.lo = r2 * (1.0f - eps);
  b.hi = r2 * (1.0f + eps);
  return b;
}

// Band for a double threshold; the conversion to float is outward-safe
// because eps covers more than one float rounding of r.
__device__ inline band make_band(double radius, float amax, int dim) {
  if (!(radius > 0.0)) {
    band b;
    b.lo = -1.0f;
    b.hi = __int_as_float(0x7f800000);
    return b;
  }
  return make_band((float) radius, amax, dim);
}

// Entry k of the kept neighbour lists (abl_near_view::ncache_list) of agent
// `self`: the neighbour's agent index.
__device__ __forceinline__ int kept_entry(const abl_near_view &V, long self, int k) {
  return V.ncache_narrow ? (int) self + (int) ABL_LDG(&((const short *) V.ncache_list)[k])
                         : ABL_LDG(&((const int *) V.ncache_list)[k]);
}

// Query side of a near loop: the agent's cell and float position.
template <int DIM>
struct near_query {
  int c[3];
  float pf[3];
  band bd;
  float amax;
  long self;  // the querying agent's index in the step's population, or -1
  // Band of the last threshold a lazy distance was compared with.
  mutable long long lazy_bits = 0;
  mutable band lazy_band;
  mutable bool lazy_valid = false;

  // `self`: the querying agent's index when it belongs to the binned
  // population (its cell is then the one binning gave it), else -1.
  __device__ near_query(const abl_near_view &V, double x, double y, double z, long self_ = -1)
      : self(self_) {
    const int dims[3] = {V.nx, V.ny, V.nz};
    const double p[3] = {x, y, z};
    if (self >= 0 && V.ncache_off) {
      c[0] = c[1] = c[2] = 0;  // kept lists: no cell search
    } else if (self >= 0 && V.cell_of) {
      const int l = (int) (ABL_LDG(&V.cell_of[self]) - V.cell_base);
      const int nxy = V.nx * V.ny;
      c[2] = l / nxy;
      c[1] = (l - c[2] * nxy) / V.nx;
      c[0] = l - c[2] * nxy - c[1] * V.nx;
    } else {
      for (int d = 0; d < 3; d++) {
        if (d >= DIM) c[d] = 0;
        else if (V.cell_f32) c[d] = cell_coord_f32((float) p[d], (float) V.lo[d], (float) V.inv_cell, dims[d]);
        else c[d] = cell_coord(p[d], V.lo[d], V.inv_cell, dims[d]);
      }
    }
    for (int d = 0; d < 3; d++) pf[d] = d < DIM ? (float) p[d] : 0.0f;
    amax = *V.amax;
    bd = make_band(V.radius, amax, DIM);
  }

  __device__ const band &band_for(double r) const {
    long long bits = __double_as_longlong(r);
    if (!lazy_valid || bits != lazy_bits) {
      lazy_band = make_band(r, amax, DIM);
      lazy_bits = bits;
      lazy_valid = true;
    }
    return lazy_band;
  }
};

// Enumerates in-radius neighbour slots in chunks of at most ABL_NEAR_CHUNK.
// `Exact` is a callable slot -> bool evaluating the reference's own test.
template <int DIM>
struct near_cursor {
  const abl_near_view &V;
  // ordered mode: position in the cell's neighbourhood list
  int cur, end;
  // unordered mode: current row of cells and slot range within it
  int rz, ry;
  int x0, x1;
  int *buf;  // this thread's column of the block's shared buffer (stride ABL_STEP_BLOCK)
  int cnt;

  __device__ int slot(int k) const { return buf[k * ABL_STEP_BLOCK]; }

  __device__ near_cursor(const abl_near_view &v, const near_query<DIM> &q) : V(v), cnt(0) {
    __shared__ int chunk[ABL_NEAR_CHUNK * ABL_STEP_BLOCK];
    buf = chunk + threadIdx.x;
    if (V.ncache_off && q.self >= 0) {
      // The agent's neighbour list kept across timesteps.
      cur = ABL_LDG(&V.ncache_off[q.self]);
      end = ABL_LDG(&V.ncache_off[q.self + 1]);
      rz = ry = 0;
      x0 = x1 = 0;
    } else if (V.ordered) {
      int cell = (q.c[2] * V.ny + q.c[1]) * V.nx + q.c[0];
      cur = V.nb_off[cell];
      end = V.nb_off[cell + 1];
    } else {
      rz = DIM == 3 ? max(q.c[2] - V.range, 0) : 0;
      ry = max(q.c[1] - V.range, 0);
      x0 = max(q.c[0] - V.range, 0);
      x1 = min(q.c[0] + V.range, V.nx - 1);
      cur = end = 0;
      row_range(q);
    }
  }

  // Loads the slot range of the current (rz, ry) row or moves past the grid.
  __device__ void row_range(const near_query<DIM> &q) {
    const int zmax = DIM == 3 ? min(q.c[2] + V.range, V.nz - 1) : 0;
    const int ymax = min(q.c[1] + V.range, V.ny - 1);
    while (rz <= zmax) {
      if (ry <= ymax) {
        int base = (rz * V.ny + ry) * V.nx;
        cur = V.cell_start[base + x0];
        end = V.cell_start[base + x1 + 1];
        return;
      }
      rz++;
      ry = max(q.c[1] - V.range, 0);
    }
    cur = end = 0;
    rz = zmax + 1;
  }

  __device__ bool exhausted(const near_query<DIM> &q) const {
    const int zmax = DIM == 3 ? min(q.c[2] + V.range, V.nz - 1) : 0;
    return rz > zmax;
  }

  template <typename Exact>
  __device__ bool fill(const near_query<DIM> &q, Exact &&exact) {
    cnt = 0;
    if (V.ncache_off && q.self >= 0) {
      while (cur < end && cnt < ABL_NEAR_CHUNK) buf[ABL_STEP_BLOCK * cnt++] = kept_entry(V, q.self, cur++);
      return cnt > 0;
    }
    for (;;) {
      while (cur < end && cnt < ABL_NEAR_CHUNK) {
        int s = V.ordered ? ABL_LDG(&V.nb_list[cur]) : cur;
        cur++;
        float d2 = 0.0f;
#pragma unroll
        for (int d = 0; d < DIM; d++) {
          float dd = ABL_LDG(&V.posf[DIM * s + d]) - q.pf[d];
          d2 = __fadd_rn(d2, __fmul_rn(dd, dd));
        }
        bool take;
        if (d2 < q.bd.lo) take = true;
        else if (d2 > q.bd.hi) take = false;
        else take = exact(s);
        if (take) buf[ABL_STEP_BLOCK * cnt++] = s;
      }
      if (cnt == ABL_NEAR_CHUNK || V.ordered) break;
      if (cur < end) break;
      // unordered: advance to the next row of cells
      if (exhausted(q)) break;
      ry++;
      row_range(q);
      if (exhausted(q)) break;
    }
    return cnt > 0;
  }
};

// ---------------------------------------------------------------------------
// Division of a double by a small positive int, bit-identical to IEEE a / n.
//
// Step bodies divide sums by neighbour counts (boids2d: the centre of the
// flock, the mean velocity, the collision centre).  FP64 is the scarce pipe
// here, and an IEEE double division is a short Newton-Raphson sequence of
// several FP64 instructions; this takes two.  Method: yh = RN(1/n) and
// yl = RN(1/n - yh) (a two-term reciprocal, |yh + yl - 1/n| <= 2^-105/n) are
// tabulated; q = RN(a*yh + RN(a*yl)) (one FMA) is a/n times (1 + e) with
// |e| <= 2^-104.  That is the correctly rounded a/n because a/n is never a
// rounding midpoint and always lies at least 2^-55/n (relative) away from
// every midpoint: with a/n in [2^E, 2^(E+1)), a - n*m is a nonzero multiple
// of 2^(E-54) for every midpoint m of that binade and the one below (a
// midpoint has a 54-bit odd significand, which n*m cannot share with the
// 53-bit a).  Needs a*yl and a/n to stay normal and finite, hence the range
// guard on a's exponent; every other case (n outside [1, kRecipN), tiny,
// huge or non-finite a) takes IEEE division.  The table is computed at
// compile time with exact arithmetic: yh by IEEE division, 1 - n*yh exactly
// from a Veltkamp split of yh (n has at most 11 bits), then one rounding.

constexpr int kRecipN = 1024;

struct alignas(16) recip_table {
  double v[2 * kRecipN];  // (yh, yl) for n = 0..kRecipN-1 (n = 0 unused)
};

constexpr double veltkamp_hi(double a) {
  const double c = 134217729.0 * a;  // 2^27 + 1
  return c - (c - a);
}

constexpr recip_table make_recip_table() {
  recip_table t{};
  for (int n = 1; n < kRecipN; n++) {
    const double yh = 1.0 / n;
    const double hi = veltkamp_hi(yh), lo = yh - hi;
    const double r = (1.0 - n * hi) - n * lo;  // 1 - n*yh, exact
    t.v[2 * n] = yh;
    t.v[2 * n + 1] = r / n;
  }
  return t;
}

static __device__ constexpr recip_table recip = make_recip_table();

__device__ __forceinline__ double div_int(double a, int n) {
  const unsigned e = ((unsigned) __double2hiint(a) >> 20) & 0x7ffu;
  if ((unsigned) (n - 1) < (unsigned) (kRecipN - 1) && e >= 200u && e < 0x7ffu) {
    const double2 y = ABL_LDG(reinterpret_cast<const double2 *>(recip.v) + n);
    return __fma_rn(a, y.x, __dmul_rn(a, y.y));
  }
  return __ddiv_rn(a, (double) n);
}

// Counter-based random numbers for random() inside step functions.  The
// reference draws from one sequential xorshift stream shared by all OpenMP
// threads (asset/c/libabl.c:8-39), which has no parallel order; here every
// draw is a pure function of (seed, agent index, step function, timestep,
// draw number): Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC'11), counter (agent, step, timestep,
// draw), key (seed low, seed high).  The CPU oracle implements the same.
struct rng {
  uint32_t k0, k1, c0, c1, c2, draw;
  // Sequential mode (abl_set_serial_random): the reference's single
  // xorshift128+ stream (asset/c/libabl.c:8-39), shared by the agents one
  // thread steps in agent order.  nullptr: the counter-based stream.
  unsigned long long *xs;

  __host__ __device__ void init(uint64_t seed, uint32_t agent, uint32_t step, uint64_t timestep) {
    k0 = (uint32_t) seed;
    k1 = (uint32_t) (seed >> 32);
    c0 = agent;
    c1 = step;
    c2 = (uint32_t) timestep;
    draw = 0;
    xs = nullptr;
  }

  // xorshift128+ (Vigna): the step the reference's xorshift128plus() takes.
  __host__ __device__ uint64_t serial_next() {
    uint64_t a = xs[0];
    const uint64_t b = xs[1];
    xs[0] = b;
    a ^= a << 23;
    xs[1] = a ^ b ^ (a >> 17) ^ (b >> 26);
    return xs[1] + b;
  }

  __host__ __device__ static void mulhilo(uint32_t a, uint32_t b, uint32_t &hi, uint32_t &lo) {
    uint64_t p = (uint64_t) a * (uint64_t) b;
    hi = (uint32_t) (p >> 32);
    lo = (uint32_t) p;
  }

  __host__ __device__ void next4(uint32_t out[4]) {
    uint32_t x0 = c0, x1 = c1, x2 = c2, x3 = draw++;
    uint32_t key0 = k0, key1 = k1;
    for (int r = 0; r < 10; r++) {
      if (r > 0) {
        key0 += 0x9E3779B9u;
        key1 += 0xBB67AE85u;
      }
      uint32_t hi0, lo0, hi1, lo1;
      mulhilo(0xD2511F53u, x0, hi0, lo0);
      mulhilo(0xCD9E8D57u, x2, hi1, lo1);
      uint32_t y0 = hi1 ^ x1 ^ key0, y2 = hi0 ^ x3 ^ key1;
      x0 = y0;
      x1 = lo1;
      x2 = y2;
      x3 = lo0;
    }
    out[0] = x0;
    out[1] = x1;
    out[2] = x2;
    out[3] = x3;
  }

  // Uniform in [0, 1) with 53 random bits.
  __host__ __device__ double unit() {
    uint32_t x[4];
    next4(x);
    uint64_t b = (((uint64_t) x[0] << 32) | x[1]) >> 11;
    return (double) b * (1.0 / 9007199254740992.0);
  }

  template <typename F>
  __host__ __device__ F uniform(F lo, F hi) {
    if (xs) {
      // random_float: min + (F) x / (F) (UINT64_MAX / (max - min)).
      const uint64_t x = serial_next();
      return lo + (F) x / (F) ((F) UINT64_MAX / (hi - lo));
    }
    F u = (F) unit();
    return lo + u * (hi - lo);
  }

  __host__ __device__ int uniform_int(int lo, int hi) {
    if (xs) {
      // random_int, with its power-of-two shortcut that omits `lo`.
      const unsigned n = (unsigned) (hi - lo + 1);
      if ((n & (n - 1)) == 0) return (int) (serial_next() & (n - 1));
      const unsigned lim = 0xffffffffu - 0xffffffffu % n;
      unsigned v;
      do {
        v = (unsigned) serial_next();
      } while (v >= lim);
      return lo + (int) (v % n);
    }
    uint32_t x[4];
    next4(x);
    uint32_t n = (uint32_t) (hi - lo) + 1u;
    return n == 0 ? (int) x[0] : lo + (int) (x[0] % n);
  }
};

// Per-thread state of a step kernel: random numbers, removeCurrent() and add().
struct step_ctx {
  rng R;
  long self;
  int removed;
  int added;
  void *const *child_cols;
  int near_col;  // presorted mode: the block agent whose neighbour list this thread reads

  __device__ void remove() { removed = 1; }
};

// Atomic max on non-negative floats (bit patterns order like the values).
__device__ inline void atomic_max_nonneg(float *addr, float v) {
  atomicMax(reinterpret_cast<int *>(addr), __float_as_int(v));
}

// ---------------------------------------------------------------------------
// Presorted mode.

// Shared memory of a presorted step kernel (dynamic, presort_bytes() at
// launch): per block agent c a column of `cap` neighbour slots and, in runs
// mode (no neighbourhood lists), their ids; then per-agent bookkeeping.
struct presort_shared {
  int *slots;            // [cap][ABL_STEP_BLOCK]: slots, ascending neighbour id
  int *ids;              // [cap][ABL_STEP_BLOCK]: runs mode, the slots' ids
  int *total;            // in-radius neighbours past the column's lower bound
  int *key;              // sort key: neighbour count, INT_MAX without agent
  int *perm;             // thread -> block agent, ascending key
  int *resume;           // lists: list index after the stored slots; rows: last stored id;
                         // block lists: block-list index after the stored slots
  int *bstart, *bend;    // block lists: the agent's cell list within `bl` (bstart -1:
                         // the column was gathered per agent)
  int *bl;               // block lists: [block_cap] slots, per cell in ascending id
  unsigned char *fresh;  // column still holds the first `cap` neighbours
  int cap;
  int block_cap;
  int mode;  // kGather*
};

// Presorted gathering modes: whole neighbourhood lists, row lists merged on
// the fly (2D), or the cells' own runs sorted per agent.
enum { kGatherRuns = 0, kGatherRows = 1, kGatherLists = 2 };

__host__ __device__ inline int gather_mode(const abl_near_view &V) {
  if (V.ncache_off) return kGatherLists;  // lists kept across timesteps: slots only
  return V.ordered ? kGatherLists : (V.rows && V.dim == 2) ? kGatherRows : kGatherRuns;
}

// Block lists reuse the column area while they are built: it must hold
// 9 ints per thread plus the scan scratch.
__host__ __device__ inline bool block_lists_fit(const abl_near_view &V) {
  return gather_mode(V) == kGatherRows && V.block_cap > 0 && V.cap >= 11;
}

__host__ __device__ inline size_t presort_bytes(const abl_near_view &V) {
  const size_t B = ABL_STEP_BLOCK;
  const size_t cols = (size_t) V.cap * B * (gather_mode(V) == kGatherRuns ? 2 : 1);
  const size_t bl = block_lists_fit(V) ? (size_t) V.block_cap : 0;
  return (cols + 6 * B + bl) * sizeof(int) + B;
}

__device__ __forceinline__ presort_shared presort_smem(const abl_near_view &V) {
  extern __shared__ int abl_presort_dyn[];
  const int B = ABL_STEP_BLOCK;
  presort_shared S;
  S.cap = V.cap;
  S.mode = gather_mode(V);
  S.slots = abl_presort_dyn;
  int *p = S.slots + S.cap * B;
  S.ids = nullptr;
  if (S.mode == kGatherRuns) {
    S.ids = p;
    p += S.cap * B;
  }
  S.total = p;
  S.key = p + B;
  S.perm = p + 2 * B;
  S.resume = p + 3 * B;
  S.bstart = p + 4 * B;
  S.bend = p + 5 * B;
  S.bl = p + 6 * B;
  S.block_cap = block_lists_fit(V) ? V.block_cap : 0;
  S.fresh = (unsigned char *) (S.bl + S.block_cap);
  return S;
}

// Runs mode: scans the candidate cells of query q and stores in column `col`
// the ids (ascending) and slots of the first S.cap in-radius neighbours with
// id > lower.  Returns how many in-radius neighbours have id > lower;
// `stored` receives how many of them the column holds.
template <int DIM, typename Exact>
__device__ int gather_sorted(const presort_shared &S, const abl_near_view &V,
                             const near_query<DIM> &q, Exact &exact, int col, int lower,
                             int &stored) {
  int *I = S.ids + col;
  int *L = S.slots + col;
  const int B = ABL_STEP_BLOCK, cap = S.cap;
  int n = 0, total = 0;
  const int zlo = DIM == 3 ? max(q.c[2] - V.range, 0) : 0;
  const int zhi = DIM == 3 ? min(q.c[2] + V.range, V.nz - 1) : 0;
  const int ylo = max(q.c[1] - V.range, 0), yhi = min(q.c[1] + V.range, V.ny - 1);
  const int x0 = max(q.c[0] - V.range, 0), x1 = min(q.c[0] + V.range, V.nx - 1);
  for (int z = zlo; z <= zhi; z++) {
    for (int y = ylo; y <= yhi; y++) {
      const int base = (z * V.ny + y) * V.nx;
      const int s1 = ABL_LDG(&V.cell_start[base + x1 + 1]);
      for (int s = ABL_LDG(&V.cell_start[base + x0]); s < s1; s++) {
        float d2 = 0.0f;
#pragma unroll
        for (int d = 0; d < DIM; d++) {
          float dd = ABL_LDG(&V.posf[DIM * s + d]) - q.pf[d];
          d2 = __fadd_rn(d2, __fmul_rn(dd, dd));
        }
        if (d2 > q.bd.hi) continue;
        const int id = ABL_LDG(&V.order[s]);
        if (id <= lower) continue;
        if (!(d2 < q.bd.lo) && !exact(s)) continue;
        total++;
        if (n == cap && id >= I[(cap - 1) * B]) continue;
        int p = n < cap ? n : cap - 1;
        while (p > 0) {
          const int prev = I[(p - 1) * B];
          if (prev < id) break;
          I[p * B] = prev;
          L[p * B] = L[(p - 1) * B];
          p--;
        }
        I[p * B] = id;
        L[p * B] = s;
        if (n < cap) n++;
      }
    }
  }
  stored = n;
  return total;
}

// Filters the candidate slots slot_at(from) .. slot_at(end - 1), which are in
// ascending id: the in-radius ones are counted and the first S.cap stored in
// column `col`; `next` receives the index after the last stored candidate.
// Four candidates are loaded at a time, so their (independent) slot and
// position loads are in flight together.
template <int DIM, typename Exact, typename SlotAt>
__device__ __forceinline__ int filter_candidates(const presort_shared &S, const abl_near_view &V,
                                                 const near_query<DIM> &q, Exact &exact,
                                                 int col, int from, int end, SlotAt slot_at,
                                                 int &stored, int &next) {
  int *L = S.slots + col;
  const int cap = S.cap;
  int n = 0, total = 0;
  next = end;
  auto consider = [&](int s, float d2, int k) {
    if (d2 > q.bd.hi) return;
    if (!(d2 < q.bd.lo) && !exact(s)) return;
    total++;
    if (n < cap) {
      L[n * ABL_STEP_BLOCK] = s;
      n++;
      if (n == cap) next = k + 1;
    }
  };
  auto dist2 = [&](int s) {
    float d2 = 0.0f;
#pragma unroll
    for (int d = 0; d < DIM; d++) {
      const float dd = ABL_LDG(&V.posf[DIM * s + d]) - q.pf[d];
      d2 = __fadd_rn(d2, __fmul_rn(dd, dd));
    }
    return d2;
  };
  int k = from;
  for (; k + 4 <= end; k += 4) {
    int sl[4];
    float d2[4];
#pragma unroll
    for (int u = 0; u < 4; u++) sl[u] = slot_at(k + u);
#pragma unroll
    for (int u = 0; u < 4; u++) d2[u] = dist2(sl[u]);
#pragma unroll
    for (int u = 0; u < 4; u++) consider(sl[u], d2[u], k + u);
  }
  for (; k < end; k++) {
    const int s = slot_at(k);
    consider(s, dist2(s), k);
  }
  stored = n;
  return total;
}

// List mode (the grid has per-cell neighbourhood lists in ascending id): from
// list index `from` on, stores the slots of the first S.cap in-radius
// neighbours in column `col` and counts all of them.  `next` receives the
// list index just past the last stored slot.
template <int DIM, typename Exact>
__device__ int gather_list(const presort_shared &S, const abl_near_view &V,
                           const near_query<DIM> &q, Exact &exact, int col, int from,
                           int &stored, int &next) {
  const int cell = (q.c[2] * V.ny + q.c[1]) * V.nx + q.c[0];
  const int end = ABL_LDG(&V.nb_off[cell + 1]);
  const int *list = V.nb_list;
  return filter_candidates(S, V, q, exact, col, from, end,
                           [list](int k) { return ABL_LDG(&list[k]); }, stored, next);
}

// Rows mode (2D): the in-radius neighbours with id > lower, taken in
// ascending id from a three-way merge of the row lists of the cells above,
// at and below the query cell.  Row list entries carry the float position
// the prefilter needs.  Stores the first S.cap slots in column `col` and
// returns how many there are in all; `last` receives the id of the last
// stored slot.
template <int DIM, typename Exact>
__device__ int gather_rows(const presort_shared &S, const abl_near_view &V,
                           const near_query<DIM> &q, Exact &exact, int col, int lower,
                           int &stored, int &last) {
  int *L = S.slots + col;
  const int cap = S.cap;
  const int kNone = 0x7fffffff;
  int pos[3], end[3];
  int4 h[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int y = q.c[1] + k - 1;
    pos[k] = end[k] = 0;
    if (y >= 0 && y < V.ny) {
      const int u = y * V.nx + q.c[0];
      pos[k] = ABL_LDG(&V.row_off[u]);
      end[k] = ABL_LDG(&V.row_off[u + 1]);
    }
    h[k] = pos[k] < end[k] ? ABL_LDG(&V.rows[pos[k]]) : make_int4(kNone, 0, 0, 0);
  }
  int n = 0, total = 0;
  last = lower;
  for (;;) {
    const bool a01 = h[0].x < h[1].x;
    const int m01 = a01 ? h[0].x : h[1].x;
    const int k = h[2].x < m01 ? 2 : (a01 ? 0 : 1);
    const int4 v = k == 0 ? h[0] : (k == 1 ? h[1] : h[2]);
    if (v.x == kNone) break;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      if (j == k) {
        const int e = ++pos[j];
        h[j] = e < end[j] ? ABL_LDG(&V.rows[e]) : make_int4(kNone, 0, 0, 0);
      }
    }
    if (v.x <= lower) continue;
    const float dx = __int_as_float(v.z) - q.pf[0], dy = __int_as_float(v.w) - q.pf[1];
    const float d2 = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
    if (d2 > q.bd.hi) continue;
    if (!(d2 < q.bd.lo) && !exact(v.y)) continue;
    total++;
    if (n < cap) {
      L[n * ABL_STEP_BLOCK] = v.y;
      n++;
      last = v.x;
    }
  }
  stored = n;
  return total;
}

// Exclusive block-wide scans of two ints (every thread of the block calls
// it; blockDim.x a multiple of 32).  `scr`: 160 ints of shared memory.
__device__ inline void block_scan2(int a, int b, int *scr, int &ea, int &eb, int &ta, int &tb) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  int ia = a, ib = b;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int xa = __shfl_up_sync(0xffffffffu, ia, o), xb = __shfl_up_sync(0xffffffffu, ib, o);
    if (lane >= o) {
      ia += xa;
      ib += xb;
    }
  }
  if (lane == 31) {
    scr[w] = ia;
    scr[32 + w] = ib;
  }
  __syncthreads();
  if (w == 0) {
    const int va = lane < nw ? scr[lane] : 0, vb = lane < nw ? scr[32 + lane] : 0;
    int sa = va, sb = vb;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int xa = __shfl_up_sync(0xffffffffu, sa, o), xb = __shfl_up_sync(0xffffffffu, sb, o);
      if (lane >= o) {
        sa += xa;
        sb += xb;
      }
    }
    scr[64 + lane] = sa - va;
    scr[96 + lane] = sb - vb;
    if (lane == 31) {
      scr[128] = sa;
      scr[129] = sb;
    }
  }
  __syncthreads();
  ea = ia - a + scr[64 + w];
  eb = ib - b + scr[96 + w];
  ta = scr[128];
  tb = scr[129];
}

// Number of ids below `id` in ids[b .. b+n) (shared memory, ascending).
__device__ __forceinline__ int ids_lower_bound(const int *ids, int b, int n, int id) {
  int lo = 0;
  while (n > 0) {
    const int half = n >> 1;
    if (ids[b + lo + half] < id) {
      lo += half + 1;
      n -= half + 1;
    } else {
      n = half;
    }
  }
  return lo;
}

// Block lists, filter: the in-radius slots of block list entries
// bl[from .. end) in order; the first S.cap go to column `col`.  Returns how
// many there are; `next` receives the entry index after the last stored one.
template <int DIM, typename Exact>
__device__ int filter_block_list(const presort_shared &S, const abl_near_view &V,
                                 const near_query<DIM> &q, Exact &exact, int col, int from,
                                 int end, int &stored, int &next) {
  const int *bl = S.bl;
  return filter_candidates(S, V, q, exact, col, from, end, [bl](int k) { return bl[k]; },
                           stored, next);
}

// Block lists (2D row lists; thread t of a block runs the agent in slot
// blockIdx.x * blockDim.x + t, so the block's agents fill a run of
// consecutive cells ca..cb, about blockDim.x / density of them).  Instead
// of every agent merging the row lists of the rows below, at and above its
// cell, the block builds each of its cells' merged list once, in shared
// memory: an entry's place in its cell's list is its index in its own row
// list plus the number of smaller ids in the other two (binary searches; the
// three lists hold different agents).  The row lists the block reads are
// those of cells ca-nx..cb-nx, ca..cb and ca+nx..cb+nx: three contiguous
// ranges of V.rows, whose ids are first copied into shared memory with
// coalesced loads, so the searches never wait on global memory.  Each thread
// then filters its cell's list.  Returns false, uniformly over the block,
// when the lists or the staged ids would not fit, the block's agents do not
// share one grid (an ensemble block spanning two replicas) or are not in
// cell order (threads not visiting slots in order); the caller then gathers
// per agent.
template <int DIM, typename Exact>
__device__ bool gather_block(const presort_shared &S, const abl_near_view &V, bool has,
                             const near_query<DIM> &q, Exact &exact, int &key) {
  const int B = ABL_STEP_BLOCK, t = threadIdx.x, nb = blockDim.x;
  // Scratch in the column area, which the filter below overwrites.
  int *cellv = S.slots;
  int *lrow = cellv + B;   // per leader thread: row list begin, 3 rows
  int *llen = lrow + 3 * B;
  int *lbase = llen + 3 * B;  // per leader ordinal: first entry of its cell's list
  int *lthr = lbase + B;      // per leader ordinal: the leader thread
  int *scr = lthr + B;        // 0..129 scans, 160..162 view check, 168..177 staging
  int *sid = scr + 192;       // staged row-list ids, to the end of the column area
  const int scap = S.cap * B - (9 * B + 192);
  const int cell = has ? q.c[1] * V.nx + q.c[0] : -1 - t;
  cellv[t] = cell;
  if (t == 0) {
    const unsigned long long vp = (unsigned long long) &V;
    scr[160] = (int) vp;
    scr[161] = (int) (vp >> 32);
    scr[162] = 0;
  }
  __syncthreads();
  {
    // One grid for the whole block, and cells in visiting order (the
    // staged ranges below hold the lists of cells cellv[0] .. the last one
    // only if no thread's cell is below its predecessor's).
    const unsigned long long vp = (unsigned long long) &V;
    if (has && (scr[160] != (int) vp || scr[161] != (int) (vp >> 32))) scr[162] = 1;
    if (has && t > 0 && cellv[t - 1] > cell) scr[162] = 1;
  }
  const bool lead = has && (t == 0 || cellv[t - 1] != cell);
  int len = 0;
  if (lead) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const int y = q.c[1] + k - 1;
      int b = 0, n = 0;
      if (y >= 0 && y < V.ny) {
        const int u = y * V.nx + q.c[0];
        b = ABL_LDG(&V.row_off[u]);
        n = ABL_LDG(&V.row_off[u + 1]) - b;
      }
      lrow[3 * t + k] = b;
      llen[3 * t + k] = n;
      len += n;
    }
  }
  int base, ord, total, nlead;
  block_scan2(len, lead ? 1 : 0, scr, base, ord, total, nlead);
  if (lead) {
    lbase[ord] = base;
    lthr[ord] = t;
  }
  if (lead && ord == nlead - 1) {
    // The last leader: stage ranges k = rows ca+(k-1)nx .. cb+(k-1)nx.
    const int ca = cellv[0], cb = cell, ncells = V.nx * V.ny;
    int staged = 0;
    for (int k = 0; k < 3; k++) {
      int lo = ca + (k - 1) * V.nx, hi = cb + (k - 1) * V.nx;
      lo = lo < 0 ? 0 : lo;
      hi = hi > ncells - 1 ? ncells - 1 : hi;
      int e0 = 0, n = 0;
      if (lo <= hi) {
        e0 = ABL_LDG(&V.row_off[lo]);
        n = ABL_LDG(&V.row_off[hi + 1]) - e0;
      }
      scr[168 + k] = e0;
      scr[171 + k] = n;
      scr[174 + k] = staged;
      staged += n;
    }
    scr[177] = staged;
  }
  __syncthreads();
  if (total > S.block_cap || scr[162] || (nlead > 0 && scr[177] > scap)) {
    __syncthreads();  // everyone has read the flags before the column is reused
    return false;
  }
  {
    const int *ids = reinterpret_cast<const int *>(V.rows);
    constexpr int kBatch = 8;
    for (int k = 0; k < 3 && nlead > 0; k++) {
      const int e0 = scr[168 + k], n = scr[171 + k], b = scr[174 + k];
      for (int i0 = 0; i0 < n; i0 += kBatch * nb) {
        int v[kBatch];
#pragma unroll
        for (int u = 0; u < kBatch; u++) {
          const int i = i0 + u * nb + t;
          if (i < n) v[u] = ABL_LDG(&ids[4 * (e0 + i)]);
        }
#pragma unroll
        for (int u = 0; u < kBatch; u++) {
          const int i = i0 + u * nb + t;
          if (i < n) sid[b + i] = v[u];
        }
      }
    }
  }
  __syncthreads();
  for (int j = t; j < total; j += nb) {
    int lo = 0, hi = nlead - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (lbase[mid] <= j) lo = mid;
      else hi = mid - 1;
    }
    const int lt = lthr[lo];
    int i = j - lbase[lo], l = 0;
    while (l < 2 && i >= llen[3 * lt + l]) {
      i -= llen[3 * lt + l];
      l++;
    }
    // Staged position of list m of this leader: its row list lies in range m.
    auto spos = [&](int m) { return scr[174 + m] + (lrow[3 * lt + m] - scr[168 + m]); };
    const int id = sid[spos(l) + i];
    const int slot = ABL_LDG(reinterpret_cast<const int *>(V.rows) + 4 * (lrow[3 * lt + l] + i) + 1);
    int p = lbase[lo] + i;
#pragma unroll
    for (int m = 0; m < 3; m++) {
      if (m != l) p += ids_lower_bound(sid, spos(m), llen[3 * lt + m], id);
    }
    S.bl[p] = slot;
  }
  // This thread's cell list: its leader is the last leader at or before it.
  const int mine = ord + (lead ? 0 : -1);
  int from = 0, end = 0;
  if (has) {
    from = lbase[mine];
    end = mine + 1 < nlead ? lbase[mine + 1] : total;
  }
  __syncthreads();  // lists complete; scratch no longer read
  if (has) {
    int stored = 0, next = 0;
    key = filter_block_list(S, V, q, exact, t, from, end, stored, next);
    S.total[t] = key;
    S.resume[t] = next;
    S.bstart[t] = from;
    S.bend[t] = end;
  }
  return true;
}

template <int DIM>
__device__ __forceinline__ int list_begin(const abl_near_view &V, const near_query<DIM> &q) {
  return ABL_LDG(&V.nb_off[(q.c[2] * V.ny + q.c[1]) * V.nx + q.c[0]]);
}

// Phase one of a presorted step kernel; every thread of the block calls it.
// Thread t gathers the neighbours of the block's agent t (has == false: no
// agent).  With V.balance set the block then ranks its agents by neighbour
// count; otherwise thread t keeps agent t.  Returns the block agent this
// thread runs the step body for.
template <int DIM, typename Exact>
__device__ int presort_block(const abl_near_view &V, bool has, const near_query<DIM> &q,
                             Exact &exact) {
  const presort_shared S = presort_smem(V);
  const int t = threadIdx.x;
  int key = 0x7fffffff;
  if (V.ncache_off) {
    // The agent's neighbour list kept across timesteps (ascending id).
    if (has) {
      const int from = ABL_LDG(&V.ncache_off[q.self]), end = ABL_LDG(&V.ncache_off[q.self + 1]);
      const int n = end - from < S.cap ? end - from : S.cap;
      for (int j = 0; j < n; j++) S.slots[j * ABL_STEP_BLOCK + t] = kept_entry(V, q.self, from + j);
      key = end - from;
      S.total[t] = key;
      S.resume[t] = from + n;
    }
  } else if (S.block_cap > 0 && gather_block(S, V, has, q, exact, key)) {
    // gathered from the block lists
  } else if (has) {
    if (S.block_cap > 0) S.bstart[t] = -1;
    int stored = 0;
    if (S.mode == kGatherLists) {
      int next = 0;
      key = gather_list(S, V, q, exact, t, list_begin(V, q), stored, next);
      S.resume[t] = next;
    } else if (S.mode == kGatherRows) {
      int last = -1;
      key = gather_rows(S, V, q, exact, t, -1, stored, last);
      S.resume[t] = last;
    } else {
      key = gather_sorted(S, V, q, exact, t, -1, stored);
    }
    S.total[t] = key;
  }
  S.fresh[t] = 1;
  if (!V.balance) return t;
  // Counting sort of the block's agents by neighbour count, in 64 buckets
  // (counts above 62 share the last; threads without an agent go last too).
  // Agents of one bucket take their places in whatever order the atomics
  // give: which thread runs an agent changes no result.
  int *hist = S.key;  // 64 counters, then bucket starts (blockDim.x >= 64)
  const int nb = blockDim.x;
  for (int i = t; i < 64; i += nb) hist[i] = 0;
  __syncthreads();
  const int b = key < 63 ? key : 63;
  const int local = atomicAdd(&hist[b], 1);
  __syncthreads();
  if (t < 32) {
    const int a = hist[2 * t], c = hist[2 * t + 1];
    int x = a + c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (t >= o) x += y;
    }
    const int start = x - a - c;
    hist[2 * t] = start;
    hist[2 * t + 1] = start + a;
  }
  __syncthreads();
  S.perm[hist[b] + local] = t;
  __syncthreads();
  return S.perm[t];
}

// Enumerates the in-radius neighbour slots of block agent `col` in ascending
// id order, in chunks of at most S.cap, starting from the column that
// presort_block left in shared memory.
template <int DIM>
struct near_list_cursor {
  const abl_near_view &V;
  const presort_shared S;
  int col;
  int cnt;
  bool first, more;
  int last;

  __device__ near_list_cursor(const abl_near_view &v, const near_query<DIM> &, const step_ctx &K)
      : V(v), S(presort_smem(v)), col(K.near_col), cnt(0), first(true), more(false), last(-1) {}

  __device__ int slot(int k) const { return S.slots[k * ABL_STEP_BLOCK + col]; }

  template <typename Exact>
  __device__ bool fill(const near_query<DIM> &q, Exact &&exact) {
    if (first && S.fresh[col]) {
      first = false;
      const int tot = S.total[col];
      cnt = tot < S.cap ? tot : S.cap;
      more = tot > S.cap;
    } else if (first || more) {
      // A second pass over the neighbours, or the ones past the stored ones.
      int stored = 0, tot = 0;
      if (V.ncache_off) {
        const int from = first ? ABL_LDG(&V.ncache_off[q.self]) : S.resume[col];
        const int end = ABL_LDG(&V.ncache_off[q.self + 1]);
        const int n = end - from < S.cap ? end - from : S.cap;
        for (int j = 0; j < n; j++) S.slots[j * ABL_STEP_BLOCK + col] = kept_entry(V, q.self, from + j);
        S.resume[col] = from + n;
        stored = n;
        tot = end - from;
      } else if (S.block_cap > 0 && S.bstart[col] >= 0) {
        const int from = first ? S.bstart[col] : S.resume[col];
        int next = 0;
        tot = filter_block_list(S, V, q, exact, col, from, S.bend[col], stored, next);
        S.resume[col] = next;
      } else if (S.mode == kGatherLists) {
        const int from = first ? list_begin(V, q) : S.resume[col];
        int next = 0;
        tot = gather_list(S, V, q, exact, col, from, stored, next);
        S.resume[col] = next;
      } else if (S.mode == kGatherRows) {
        int lastid = -1;
        tot = gather_rows(S, V, q, exact, col, first ? -1 : S.resume[col], stored, lastid);
        S.resume[col] = lastid;
      } else {
        tot = gather_sorted(S, V, q, exact, col, first ? -1 : last, stored);
      }
      first = false;
      S.fresh[col] = 0;
      cnt = stored;
      more = tot > stored;
    } else {
      cnt = 0;
    }
    if (cnt > 0 && S.mode == kGatherRuns) last = S.ids[(cnt - 1) * ABL_STEP_BLOCK + col];
    return cnt > 0;
  }
};

// A distance between the query agent and the current neighbour that the
// generated code only ever compares with loop-invariant values, e.g.
//   float separation = dist(in.pos, nx.pos); if (separation < R) ...
// A comparison is decided from the FP32 estimate whenever it lies outside the
// error band of make_band(R); otherwise the reference expression (`exact`)
// is evaluated.  Either way the result equals the reference's comparison.
template <int DIM, typename Exact>
struct lazy_dist {
  const near_query<DIM> &q;
  float d2f;
  Exact exact;

  __device__ lazy_dist(const near_query<DIM> &q_, const abl_near_view &V, int slot, Exact e)
      : q(q_), exact(e) {
    float d2 = 0.0f;
#pragma unroll
    for (int d = 0; d < DIM; d++) {
      float dd = ABL_LDG(&V.posf[DIM * slot + d]) - q.pf[d];
      d2 = __fadd_rn(d2, __fmul_rn(dd, dd));
    }
    d2f = d2;
  }

  // -1: surely below R, +1: surely above R, 0: undecided.
  __device__ int side(double R) const {
    const band &b = q.band_for(R);
    if (d2f < b.lo) return -1;
    if (d2f > b.hi) return 1;
    return 0;
  }
};

template <int DIM, typename Exact>
__device__ lazy_dist<DIM, Exact> make_lazy_dist(const near_query<DIM> &q, const abl_near_view &V,
                                                int slot, Exact e) {
  return lazy_dist<DIM, Exact>(q, V, slot, e);
}

template <int DIM, typename Exact, typename R>
__device__ inline bool operator<(const lazy_dist<DIM, Exact> &a, R r) {
  int s = a.side((double) r);
  return s < 0 ? true : s > 0 ? false : a.exact() < r;
}
template <int DIM, typename Exact, typename R>
__device__ inline bool operator<=(const lazy_dist<DIM, Exact> &a, R r) {
  int s = a.side((double) r);
  return s < 0 ? true : s > 0 ? false : a.exact() <= r;
}
template <int DIM, typename Exact, typename R>
__device__ inline bool operator>(const lazy_dist<DIM, Exact> &a, R r) {
  int s = a.side((double) r);
  return s < 0 ? false : s > 0 ? true : a.exact() > r;
}
template <int DIM, typename Exact, typename R>
__device__ inline bool operator>=(const lazy_dist<DIM, Exact> &a, R r) {
  int s = a.side((double) r);
  return s < 0 ? false : s > 0 ? true : a.exact() >= r;
}
template <int DIM, typename Exact, typename R>
__device__ inline bool operator==(const lazy_dist<DIM, Exact> &a, R r) {
  int s = a.side((double) r);
  return s != 0 ? false : a.exact() == r;
}
template <int DIM, typename Exact, typename R>
__device__ inline bool operator!=(const lazy_dist<DIM, Exact> &a, R r) {
  int s = a.side((double) r);
  return s != 0 ? true : a.exact() != r;
}
// R OP d  is  d OP' R.
template <int DIM, typename Exact, typename R>
__device__ inline bool operator<(R r, const lazy_dist<DIM, Exact> &a) { return a > r; }
template <int DIM, typename Exact, typename R>
__device__ inline bool operator<=(R r, const lazy_dist<DIM, Exact> &a) { return a >= r; }
template <int DIM, typename Exact, typename R>
__device__ inline bool operator>(R r, const lazy_dist<DIM, Exact> &a) { return a < r; }
template <int DIM, typename Exact, typename R>
__device__ inline bool operator>=(R r, const lazy_dist<DIM, Exact> &a) { return a <= r; }
template <int DIM, typename Exact, typename R>
__device__ inline bool operator==(R r, const lazy_dist<DIM, Exact> &a) { return a == r; }
template <int DIM, typename Exact, typename R>
__device__ inline bool operator!=(R r, const lazy_dist<DIM, Exact> &a) { return a != r; }

// ------------------------------------------------ mixed precision (-C cuda.precision=mixed)
//
// A near-loop accumulation `acc += nx.m` of a floating-point member runs in
// FP32 in the mixed form; everything else (the radius test, the body's other
// arithmetic, the step's integration) stays FP64.
//  - m the position: the sum of offsets from the querying position p,
//    (nx.pos - p), each formed from the neighbour's position split in two
//    floats (hi = (float) pos, lo = (float) (pos - hi), slot-ordered copies
//    made by the binning) minus p split the same way; after the loop
//    acc += n * p + sum.  The offsets are short (within the radius), so
//    their FP32 sum keeps ~2^-24 of the radius, not of the coordinates.
//  - another member: the FP32 sum of its float copy; after the loop
//    acc += sum.

template <int DIM>
struct mixed_anchor {
  double p[3];
  float hi[3], lo[3];
  __device__ mixed_anchor(double x, double y, double z) {
    const double q[3] = {x, y, z};
#pragma unroll
    for (int d = 0; d < 3; d++) {
      p[d] = d < DIM ? q[d] : 0.0;
      hi[d] = (float) p[d];
      lo[d] = (float) (p[d] - (double) hi[d]);
    }
  }
};

template <int DIM>
struct facc {
  float v[DIM];
  int n;
  __device__ facc() : n(0) {
#pragma unroll
    for (int d = 0; d < DIM; d++) v[d] = 0.0f;
  }
  // += (position of slot s) - anchor
  // DIM floats of a slot-ordered array (one 8-byte load for two)
  __device__ __forceinline__ static void load(const float *a, int s, float *out) {
    if (DIM == 2) {
      const ::float2 t = ABL_LDG(reinterpret_cast<const ::float2 *>(a) + s);
      out[0] = t.x;
      out[DIM - 1] = t.y;
    } else {
#pragma unroll
      for (int d = 0; d < DIM; d++) out[d] = ABL_LDG(&a[DIM * s + d]);
    }
  }
  __device__ __forceinline__ void add_offset(const abl_near_view &V, int s,
                                             const mixed_anchor<DIM> &a) {
    float ph[DIM], pl[DIM];
    load(V.posf, s, ph);
    load(V.poslo, s, pl);
#pragma unroll
    for (int d = 0; d < DIM; d++) {
      const float hi = __fsub_rn(ph[d], a.hi[d]);
      const float lo = __fsub_rn(pl[d], a.lo[d]);
      v[d] = __fadd_rn(v[d], __fadd_rn(hi, lo));
    }
    n++;
  }
  // += float copy of member column `k` at slot s (DIM components)
  __device__ __forceinline__ void add_member(const abl_near_view &V, int k, int s) {
    float m[DIM];
    load((const float *) V.fcols[k], s, m);
#pragma unroll
    for (int d = 0; d < DIM; d++) v[d] = __fadd_rn(v[d], m[d]);
    n++;
  }
  // The accumulated value in FP64: n * anchor + offsets, or the plain sum.
  __device__ __forceinline__ double offset_total(const mixed_anchor<DIM> &a, int d) const {
    return a.p[d] * (double) n + (double) v[d];
  }
  __device__ __forceinline__ double total(int d) const { return (double) v[d]; }
};

}  // namespace abl
