/* CPU oracle for the OpenABL `near()` hot path — TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C, what the reference `c` backend emits for
 * the example models (src/backend/CPrinter.cpp, GenericPrinter.cpp,
 * GenericCPrinter.cpp) together with the arithmetic of the reference runtime
 * (asset/c/libabl.h, asset/c/libabl.c).  Only the test suite, the smoke check
 * and the CPU-baseline leg of the benchmark load it, as the checker or as the
 * timed CPU baseline; the CUDA product path never calls it.
 *
 * Parity pin: the brute-force mode of every model here is checked, step by
 * step, against dumps of the reference programs themselves (the reference
 * compiler's `c` output built with the reference libabl.c), stored as golden
 * hashes under tests/golden/ by tests/golden/make_golden.py.
 *
 * Arithmetic rules restated from the reference (and required for bit
 * equality):
 *  - abl_float is double (float under LIBABL_USE_FLOAT), libabl.h:59-63;
 *  - float2/float3 ops are component-wise +,-,*,/ (libabl.h:80-143);
 *  - length/dist take sqrtf of the double sum of squares, i.e. the sum is
 *    rounded to float before the square root (libabl.h:156-168);
 *  - no FMA contraction (gcc -std=c99 defaults to -ffp-contract=off; this
 *    file is compiled with -ffp-contract=off explicitly);
 *  - the near loop visits every agent of the neighbour type in ascending
 *    index, the agent itself included, and skips it when
 *    dist(nx.pos, in.pos) > radius (CPrinter.cpp:148-173);
 *  - reads come from the current buffer and writes go to the double buffer
 *    (CPrinter.cpp:189-233).
 *
 * Two neighbour-search modes give identical results:
 *  - mode 0 (brute force) is the reference loop itself, O(N^2);
 *  - mode 1 (binned) buckets agents into a uniform grid whose cells are 1%
 *    wider than the radius, gathers the candidates of the 3x3 (3x3x3) cells
 *    around each agent, sorts them by index and runs the same test and body
 *    in that order.  A pair that passes the float-rounded radius test is at
 *    most a few float ulps beyond the radius, far inside the 1% margin, so no
 *    passing neighbour is missed and the visiting order is unchanged.
 */
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_API __attribute__((visibility("default")))

/* ------------------------------------------------------------------ RNG */
/* xorshift128+ with the fixed seed of asset/c/libabl.c:8-17. */

static uint64_t xs_state[2] = {0xdeadbeef, 0xbeefdead};

static uint64_t xs_next(void) {
  uint64_t x = xs_state[0];
  uint64_t const y = xs_state[1];
  xs_state[0] = y;
  x ^= x << 23;
  xs_state[1] = x ^ y ^ (x >> 17) ^ (y >> 26);
  return xs_state[1] + y;
}

ORACLE_API void oracle_rng_reset(void) {
  xs_state[0] = 0xdeadbeef;
  xs_state[1] = 0xbeefdead;
}

/* random_float, asset/c/libabl.c:19-24 (FP64 build). */
ORACLE_API double oracle_random_float(double min, double max) {
  uint64_t x = xs_next();
  return min + (double) x / (double) (UINT64_MAX / (max - min));
}

/* random_int, asset/c/libabl.c:26-39, including its power-of-two shortcut
 * that ignores `min`. */
ORACLE_API int oracle_random_int(int min, int max) {
  unsigned n = max - min + 1;
  if ((n & (n - 1)) == 0) {
    return (int) (xs_next() & (n - 1));
  }
  unsigned r = UINT_MAX % n;
  unsigned x;
  do {
    x = (unsigned) xs_next();
  } while (x >= UINT_MAX - r);
  return min + x % n;
}

/* --------------------------------------------------------- reference init
 * The examples' main() bodies draw agents sequentially.  The reference
 * prints random(float2 min, float2 max) as
 *   float2_create(random_float(min.x, max.x), random_float(min.y, max.y))
 * (asset/lib.abl:14-19 through GenericPrinter).  C leaves the evaluation
 * order of those arguments unspecified; the reference programs built with
 * gcc 13 on x86-64 draw the LAST component first, and so do these
 * restatements, so that they reproduce the reference's initial states. */

static void draw_vec(double *out, int dim, const double *lo, const double *hi) {
  for (int d = dim - 1; d >= 0; d--) out[d] = oracle_random_float(lo[d], hi[d]);
}

/* examples/circle.abl:59-66 and examples/circle3d.abl:59-66:
 * pos = random(float2(W)) (random(environment.max) in 3D). */
ORACLE_API void oracle_init_circle(int dim, long n, double W, double *pos) {
  double lo[3] = {0, 0, 0}, hi[3] = {W, W, W};
  for (long i = 0; i < n; i++) draw_vec(pos + dim * i, dim, lo, hi);
}

/* examples/boids2d.abl:110-118: pos = random(float2(min_pos), float2(max_pos)),
 * velocity = random(float2(-1), float2(1)); the compound literal's members
 * are drawn in declaration order. */
ORACLE_API void oracle_init_boids2d(long n, double min_pos, double max_pos, double *pos,
                                    double *vel) {
  double plo[2] = {min_pos, min_pos}, phi[2] = {max_pos, max_pos};
  double vlo[2] = {-1, -1}, vhi[2] = {1, 1};
  for (long i = 0; i < n; i++) {
    draw_vec(pos + 2 * i, 2, plo, phi);
    draw_vec(vel + 2 * i, 2, vlo, vhi);
  }
}

/* examples/game_of_life.abl:63-75 with debug = false:
 * pos = float2(x + 0.5, y + 0.5) (x cast to C float first, as the reference
 * prints `(float) x`), alive = random(0, 1) < alive_fraction. */
ORACLE_API void oracle_init_game_of_life(int size, double alive_fraction, double *pos,
                                         uint8_t *alive) {
  long i = 0;
  for (int x = 0; x < size; ++x) {
    for (int y = 0; y < size; ++y, ++i) {
      pos[2 * i] = (double) ((float) x) + 0.5;
      pos[2 * i + 1] = (double) ((float) y) + 0.5;
      alive[i] = oracle_random_float(0, 1) < alive_fraction;
    }
  }
}

/* --------------------------------------------------------- vector math */

static inline double dist2(const double *a, const double *b) {
  /* dist_float2: sqrtf((a-b).x^2 + (a-b).y^2), libabl.h:156,164 */
  double dx = a[0] - b[0], dy = a[1] - b[1];
  return (double) sqrtf((float) (dx * dx + dy * dy));
}

static inline double dist3(const double *a, const double *b) {
  /* dist_float3, libabl.h:159,167 */
  double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
  return (double) sqrtf((float) (dx * dx + dy * dy + dz * dz));
}

static inline double distd(int dim, const double *a, const double *b) {
  return dim == 2 ? dist2(a, b) : dist3(a, b);
}

/* -------------------------------------------------------------- binning */

typedef struct {
  int dim;
  long n;
  long dims[3];
  double lo[3];
  double inv_cell;
  long *cell_start; /* ncells + 1 */
  long *order;      /* agent indices sorted by (cell, index) */
  long *cell_of;    /* cell of every agent */
} grid_t;

static long clampl(long v, long lo, long hi) { return v < lo ? lo : v > hi ? hi : v; }

static void grid_build(grid_t *g, int dim, long n, const double *pos, const double *env_min,
                       const double *env_max, double radius) {
  double cell = radius * 1.01;
  g->dim = dim;
  g->n = n;
  g->inv_cell = 1.0 / cell;
  long ncells = 1;
  for (int d = 0; d < 3; d++) {
    if (d < dim) {
      g->lo[d] = env_min[d];
      long k = (long) floor((env_max[d] - env_min[d]) * g->inv_cell) + 1;
      g->dims[d] = k < 1 ? 1 : k;
    } else {
      g->lo[d] = 0;
      g->dims[d] = 1;
    }
    ncells *= g->dims[d];
  }
  g->cell_start = calloc(ncells + 1, sizeof(long));
  g->order = malloc((n ? n : 1) * sizeof(long));
  g->cell_of = malloc((n ? n : 1) * sizeof(long));
  for (long i = 0; i < n; i++) {
    long c = 0;
    for (int d = dim - 1; d >= 0; d--) {
      long k = (long) floor((pos[dim * i + d] - g->lo[d]) * g->inv_cell);
      c = c * g->dims[d] + clampl(k, 0, g->dims[d] - 1);
    }
    g->cell_of[i] = c;
    g->cell_start[c + 1]++;
  }
  for (long c = 0; c < ncells; c++) g->cell_start[c + 1] += g->cell_start[c];
  long *fill = malloc((ncells + 1) * sizeof(long));
  memcpy(fill, g->cell_start, (ncells + 1) * sizeof(long));
  for (long i = 0; i < n; i++) g->order[fill[g->cell_of[i]]++] = i; /* stable */
  free(fill);
}

static void grid_free(grid_t *g) {
  free(g->cell_start);
  free(g->order);
  free(g->cell_of);
}

static int cmp_long(const void *a, const void *b) {
  long x = *(const long *) a, y = *(const long *) b;
  return x < y ? -1 : x > y;
}

/* Candidates of agent i: all agents in the 3^dim cells around its cell,
 * returned in ascending index order.  `buf` grows as needed. */
static long grid_candidates(const grid_t *g, long i, long **buf, long *cap) {
  long c = g->cell_of[i];
  long k[3] = {0, 0, 0};
  long rem = c;
  for (int d = 0; d < g->dim; d++) {
    k[d] = rem % g->dims[d];
    rem /= g->dims[d];
  }
  long cnt = 0;
  long z0 = g->dim == 3 ? k[2] - 1 : 0, z1 = g->dim == 3 ? k[2] + 1 : 0;
  for (long z = z0; z <= z1; z++) {
    if (z < 0 || z >= g->dims[2]) continue;
    for (long y = k[1] - 1; y <= k[1] + 1; y++) {
      if (y < 0 || y >= g->dims[1]) continue;
      for (long x = k[0] - 1; x <= k[0] + 1; x++) {
        if (x < 0 || x >= g->dims[0]) continue;
        long cc = (z * g->dims[1] + y) * g->dims[0] + x;
        long s = g->cell_start[cc], e = g->cell_start[cc + 1];
        if (cnt + (e - s) > *cap) {
          *cap = 2 * (cnt + (e - s)) + 64;
          *buf = realloc(*buf, *cap * sizeof(long));
        }
        for (long j = s; j < e; j++) (*buf)[cnt++] = g->order[j];
      }
    }
  }
  qsort(*buf, cnt, sizeof(long), cmp_long);
  return cnt;
}

/* Iterates the neighbour candidates of agent i in ascending index order:
 * every agent in brute-force mode, the sorted grid candidates otherwise. */
#define FOR_EACH_CANDIDATE(j, i, n, mode, grid, buf, cap, ...)               \
  do {                                                                       \
    if ((mode) == 0) {                                                       \
      for (long j = 0; j < (n); j++) { __VA_ARGS__ }                                \
    } else {                                                                 \
      long cnt_ = grid_candidates((grid), (i), &(buf), &(cap));              \
      for (long q_ = 0; q_ < cnt_; q_++) { long j = (buf)[q_]; __VA_ARGS__ }        \
    }                                                                        \
  } while (0)

static int threads_or_default(int nthreads) {
#ifdef _OPENMP
  return nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  (void) nthreads;
  return 1;
#endif
}

/* ------------------------------------------------------------ circle */
/* examples/circle.abl:41-57 (dim 2) and examples/circle3d.abl:41-57 (dim 3),
 * as printed by the reference:
 *   new_pos = in.pos
 *   for nx near(in, 2*r) [skip if dist(nx.pos, in.pos) > (2.0 * r)]:
 *     pos_dist = dist(in.pos, nx.pos); if (pos_dist == 0) continue;
 *     sep_dist = pos_dist - r; force = fill(0)
 *     if (sep_dist > 0.0)
 *       force = ((nx.pos - in.pos) * (k_att * ((2.0 * r) - pos_dist))) / pos_dist
 *     else force = (in.pos - nx.pos) * k_rep
 *     new_pos = new_pos + force
 *   out.pos = clamp(new_pos, fill(1), fill(W - 1.0))
 * (scalar * vector is normalised to vector * scalar by the analysis,
 * src/AnalysisVisitor.cpp:971-974; clamp is asset/lib.abl:54-67).
 * `first`/`count` select the agents whose step is computed (a bounded sample
 * for CPU timing); pass 0 and n for the whole population. */
ORACLE_API int oracle_circle_step(int dim, long n, const double *pos_in, double *pos_out,
                                  double r, double k_rep, double k_att, double W,
                                  const double *env_min, const double *env_max, int mode,
                                  int nthreads, long first, long count) {
  grid_t g;
  double radius = 2.0 * r;
  if (mode == 1) grid_build(&g, dim, n, pos_in, env_min, env_max, radius);
#pragma omp parallel num_threads(threads_or_default(nthreads))
  {
    long *buf = NULL, cap = 0;
#pragma omp for schedule(dynamic, 64)
    for (long i = first; i < first + count; i++) {
      const double *ip = pos_in + dim * i;
      double new_pos[3] = {ip[0], ip[1], dim == 3 ? ip[2] : 0};
      FOR_EACH_CANDIDATE(j, i, n, mode, &g, buf, cap, {
        const double *jp = pos_in + dim * j;
        if (distd(dim, jp, ip) > radius) continue;
        double pos_dist = distd(dim, ip, jp);
        if (pos_dist == 0) continue;
        double sep_dist = pos_dist - r;
        double force[3] = {0, 0, 0};
        if (sep_dist > 0.0) {
          double s = k_att * ((2.0 * r) - pos_dist);
          for (int d = 0; d < dim; d++) force[d] = ((jp[d] - ip[d]) * s) / pos_dist;
        } else {
          for (int d = 0; d < dim; d++) force[d] = (ip[d] - jp[d]) * k_rep;
        }
        for (int d = 0; d < dim; d++) new_pos[d] = new_pos[d] + force[d];
      });
      double lo = 1, hi = W - 1.0;
      for (int d = 0; d < dim; d++) {
        double p = new_pos[d];
        pos_out[dim * i + d] = (p < lo) ? lo : ((p > hi) ? hi : p);
      }
    }
    free(buf);
  }
  if (mode == 1) grid_free(&g);
  return 0;
}

/* ------------------------------------------------------------ boids2d */
/* examples/boids2d.abl:43-108 as printed by the reference (see the module
 * comment for the arithmetic rules).  Parameters are the printed constants:
 * p[0..9] = interaction_radius, separation_radius, time_scale, global_scale,
 * steer_scale, collision_scale, match_scale, min_pos, max_pos, (unused). */
ORACLE_API int oracle_boids2d_step(long n, const double *pos_in, const double *vel_in,
                                   double *pos_out, double *vel_out, const double *p,
                                   int mode, int nthreads, long first, long count) {
  const double interaction_radius = p[0], separation_radius = p[1], time_scale = p[2],
               global_scale = p[3], steer_scale = p[4], collision_scale = p[5],
               match_scale = p[6], min_pos = p[7], max_pos = p[8];
  grid_t g;
  double emin[2] = {min_pos, min_pos}, emax[2] = {max_pos, max_pos};
  if (mode == 1) grid_build(&g, 2, n, pos_in, emin, emax, interaction_radius);
#pragma omp parallel num_threads(threads_or_default(nthreads))
  {
    long *buf = NULL, cap = 0;
#pragma omp for schedule(dynamic, 64)
    for (long i = first; i < first + count; i++) {
      const double *ip = pos_in + 2 * i;
      const double *iv = vel_in + 2 * i;
      double gv[2] = {0, 0}, gc[2] = {0, 0}, cc[2] = {0, 0};
      int interaction_count = 0, collision_count = 0;
      FOR_EACH_CANDIDATE(j, i, n, mode, &g, buf, cap, {
        const double *jp = pos_in + 2 * j;
        const double *jv = vel_in + 2 * j;
        if (dist2(jp, ip) > interaction_radius) continue;
        gc[0] = gc[0] + jp[0];
        gc[1] = gc[1] + jp[1];
        gv[0] = gv[0] + jv[0];
        gv[1] = gv[1] + jv[1];
        interaction_count += 1;
        double separation = dist2(ip, jp);
        if (separation < separation_radius) {
          cc[0] = cc[0] + jp[0];
          cc[1] = cc[1] + jp[1];
          collision_count += 1;
        }
      });
      double vc[2] = {0, 0};
      double steer[2] = {0, 0};
      if (interaction_count > 0) {
        gc[0] = gc[0] / interaction_count;
        gc[1] = gc[1] / interaction_count;
        steer[0] = (gc[0] - ip[0]) * steer_scale;
        steer[1] = (gc[1] - ip[1]) * steer_scale;
      }
      vc[0] = vc[0] + steer[0];
      vc[1] = vc[1] + steer[1];
      double match[2] = {0, 0};
      if (interaction_count > 0) {
        gv[0] = gv[0] / interaction_count;
        gv[1] = gv[1] / interaction_count;
        match[0] = gv[0] * match_scale;
        match[1] = gv[1] * match_scale;
      }
      vc[0] = vc[0] + match[0];
      vc[1] = vc[1] + match[1];
      double avoid[2] = {0, 0};
      if (collision_count > 0) {
        cc[0] = cc[0] / collision_count;
        cc[1] = cc[1] / collision_count;
        avoid[0] = (ip[0] - cc[0]) * collision_scale;
        avoid[1] = (ip[1] - cc[1]) * collision_scale;
      }
      vc[0] = vc[0] + avoid[0];
      vc[1] = vc[1] + avoid[1];
      double nv[2] = {iv[0] + vc[0] * global_scale, iv[1] + vc[1] * global_scale};
      double scale = (double) sqrtf((float) (nv[0] * nv[0] + nv[1] * nv[1]));
      if (scale > 1) {
        nv[0] = nv[0] / scale;
        nv[1] = nv[1] / scale;
      }
      double np[2] = {ip[0] + nv[0] * time_scale, ip[1] + nv[1] * time_scale};
      /* boundPosition, examples/boids2d.abl:43-50 */
      for (int d = 0; d < 2; d++) {
        double v = np[d];
        np[d] = v < min_pos ? max_pos : (v > max_pos ? min_pos : v);
      }
      pos_out[2 * i] = np[0];
      pos_out[2 * i + 1] = np[1];
      vel_out[2 * i] = nv[0];
      vel_out[2 * i + 1] = nv[1];
    }
    free(buf);
  }
  if (mode == 1) grid_free(&g);
  return 0;
}

/* ------------------------------------------------------- game of life */
/* examples/game_of_life.abl:45-61 as printed by the reference:
 *   living = 0; for nx near(in, radius): living += nx.alive ? 1 : 0
 *   if (in.alive) { living -= 1; out.alive = living >= 2 && living <= 3 }
 *   else out.alive = living == 3
 *   out.pos = in.pos */
ORACLE_API int oracle_game_of_life_step(long n, const double *pos_in, const uint8_t *alive_in,
                                        double *pos_out, uint8_t *alive_out, double radius,
                                        double size, int mode, int nthreads, long first,
                                        long count) {
  grid_t g;
  double emin[2] = {0, 0}, emax[2] = {size, size};
  if (mode == 1) grid_build(&g, 2, n, pos_in, emin, emax, radius);
#pragma omp parallel num_threads(threads_or_default(nthreads))
  {
    long *buf = NULL, cap = 0;
#pragma omp for schedule(dynamic, 256)
    for (long i = first; i < first + count; i++) {
      const double *ip = pos_in + 2 * i;
      int living = 0;
      FOR_EACH_CANDIDATE(j, i, n, mode, &g, buf, cap, {
        if (dist2(pos_in + 2 * j, ip) > radius) continue;
        living += alive_in[j] ? 1 : 0;
      });
      if (alive_in[i]) {
        living -= 1;
        alive_out[i] = (living >= 2) && (living <= 3);
      } else {
        alive_out[i] = living == 3;
      }
      pos_out[2 * i] = ip[0];
      pos_out[2 * i + 1] = ip[1];
    }
    free(buf);
  }
  if (mode == 1) grid_free(&g);
  return 0;
}
