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

/* examples/boids.abl:112-120 (3D): pos = random(float3(min_pos), float3(max_pos)),
 * velocity = random(float3(-1), float3(1)). */
ORACLE_API void oracle_init_boids3d(long n, double min_pos, double max_pos, double *pos,
                                    double *vel) {
  double plo[3] = {min_pos, min_pos, min_pos}, phi[3] = {max_pos, max_pos, max_pos};
  double vlo[3] = {-1, -1, -1}, vhi[3] = {1, 1, 1};
  for (long i = 0; i < n; i++) {
    draw_vec(pos + 3 * i, 3, plo, phi);
    draw_vec(vel + 3 * i, 3, vlo, vhi);
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

/* ------------------------------------------------------------ boids */
/* examples/boids2d.abl:43-108 (DIM 2) and examples/boids.abl:43-110 (DIM 3,
 * the same rules on float3) as printed by the reference (see the module
 * comment for the arithmetic rules).  Parameters are the printed constants:
 * p[0..9] = interaction_radius, separation_radius, time_scale, global_scale,
 * steer_scale, collision_scale, match_scale, min_pos, max_pos, (unused).
 * Component-wise statements keep the reference's order of operations; length
 * and dist sum the squares x, y, z left to right (libabl.h:156-167). */
static int boids_step(int dim, long n, const double *pos_in, const double *vel_in,
                      double *pos_out, double *vel_out, const double *p, int mode, int nthreads,
                      long first, long count) {
  const double interaction_radius = p[0], separation_radius = p[1], time_scale = p[2],
               global_scale = p[3], steer_scale = p[4], collision_scale = p[5],
               match_scale = p[6], min_pos = p[7], max_pos = p[8];
  grid_t g;
  double emin[3] = {min_pos, min_pos, min_pos}, emax[3] = {max_pos, max_pos, max_pos};
  if (mode == 1) grid_build(&g, dim, n, pos_in, emin, emax, interaction_radius);
#pragma omp parallel num_threads(threads_or_default(nthreads))
  {
    long *buf = NULL, cap = 0;
#pragma omp for schedule(dynamic, 64)
    for (long i = first; i < first + count; i++) {
      const double *ip = pos_in + dim * i;
      const double *iv = vel_in + dim * i;
      double gv[3] = {0, 0, 0}, gc[3] = {0, 0, 0}, cc[3] = {0, 0, 0};
      int interaction_count = 0, collision_count = 0;
      FOR_EACH_CANDIDATE(j, i, n, mode, &g, buf, cap, {
        const double *jp = pos_in + dim * j;
        const double *jv = vel_in + dim * j;
        if (distd(dim, jp, ip) > interaction_radius) continue;
        for (int d = 0; d < dim; d++) gc[d] = gc[d] + jp[d];
        for (int d = 0; d < dim; d++) gv[d] = gv[d] + jv[d];
        interaction_count += 1;
        double separation = distd(dim, ip, jp);
        if (separation < separation_radius) {
          for (int d = 0; d < dim; d++) cc[d] = cc[d] + jp[d];
          collision_count += 1;
        }
      });
      double vc[3] = {0, 0, 0};
      double steer[3] = {0, 0, 0};
      if (interaction_count > 0) {
        for (int d = 0; d < dim; d++) gc[d] = gc[d] / interaction_count;
        for (int d = 0; d < dim; d++) steer[d] = (gc[d] - ip[d]) * steer_scale;
      }
      for (int d = 0; d < dim; d++) vc[d] = vc[d] + steer[d];
      double match[3] = {0, 0, 0};
      if (interaction_count > 0) {
        for (int d = 0; d < dim; d++) gv[d] = gv[d] / interaction_count;
        for (int d = 0; d < dim; d++) match[d] = gv[d] * match_scale;
      }
      for (int d = 0; d < dim; d++) vc[d] = vc[d] + match[d];
      double avoid[3] = {0, 0, 0};
      if (collision_count > 0) {
        for (int d = 0; d < dim; d++) cc[d] = cc[d] / collision_count;
        for (int d = 0; d < dim; d++) avoid[d] = (ip[d] - cc[d]) * collision_scale;
      }
      for (int d = 0; d < dim; d++) vc[d] = vc[d] + avoid[d];
      double nv[3] = {0, 0, 0};
      for (int d = 0; d < dim; d++) nv[d] = iv[d] + vc[d] * global_scale;
      double ss = nv[0] * nv[0] + nv[1] * nv[1];
      if (dim == 3) ss = ss + nv[2] * nv[2];
      double scale = (double) sqrtf((float) ss);
      if (scale > 1) {
        for (int d = 0; d < dim; d++) nv[d] = nv[d] / scale;
      }
      /* boundPosition (examples/boids2d.abl:43-50, boids.abl:43-52) */
      for (int d = 0; d < dim; d++) {
        double v = ip[d] + nv[d] * time_scale;
        pos_out[dim * i + d] = v < min_pos ? max_pos : (v > max_pos ? min_pos : v);
        vel_out[dim * i + d] = nv[d];
      }
    }
    free(buf);
  }
  if (mode == 1) grid_free(&g);
  return 0;
}

ORACLE_API int oracle_boids2d_step(long n, const double *pos_in, const double *vel_in,
                                   double *pos_out, double *vel_out, const double *p,
                                   int mode, int nthreads, long first, long count) {
  return boids_step(2, n, pos_in, vel_in, pos_out, vel_out, p, mode, nthreads, first, count);
}

ORACLE_API int oracle_boids3d_step(long n, const double *pos_in, const double *vel_in,
                                   double *pos_out, double *vel_out, const double *p,
                                   int mode, int nthreads, long first, long count) {
  return boids_step(3, n, pos_in, vel_in, pos_out, vel_out, p, mode, nthreads, first, count);
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

/* ----------------------------------------------------- boids2d (FP32) */
/* examples/boids2d.abl:43-108 as the reference builds it with
 * LIBABL_USE_FLOAT (-C use_float=true): abl_float is float, so agents,
 * globals and every float2 operation of libabl.h are single precision;
 * length/dist are sqrtf of the float sum of squares.  Parameters as for
 * oracle_boids2d_step, rounded to float as the printed `float` globals are.
 * Positions are widened to double for the candidate grid only. */
static inline float dist2f(const float *a, const float *b) {
  const float dx = a[0] - b[0], dy = a[1] - b[1];
  return sqrtf(dx * dx + dy * dy);
}

ORACLE_API int oracle_boids2d_step_f32(long n, const float *pos_in, const float *vel_in,
                                       float *pos_out, float *vel_out, const float *p,
                                       int mode, int nthreads) {
  const float interaction_radius = p[0], separation_radius = p[1], time_scale = p[2],
              global_scale = p[3], steer_scale = p[4], collision_scale = p[5],
              match_scale = p[6], min_pos = p[7], max_pos = p[8];
  grid_t g;
  double *posd = NULL;
  if (mode == 1) {
    posd = (double *) malloc(sizeof(double) * 2 * (n > 0 ? n : 1));
    for (long k = 0; k < 2 * n; k++) posd[k] = pos_in[k];
    double emin[2] = {min_pos, min_pos}, emax[2] = {max_pos, max_pos};
    grid_build(&g, 2, n, posd, emin, emax, interaction_radius);
  }
#pragma omp parallel num_threads(threads_or_default(nthreads))
  {
    long *buf = NULL, cap = 0;
#pragma omp for schedule(dynamic, 64)
    for (long i = 0; i < n; i++) {
      const float *ip = pos_in + 2 * i;
      const float *iv = vel_in + 2 * i;
      float gv[2] = {0, 0}, gc[2] = {0, 0}, cc[2] = {0, 0};
      int interaction_count = 0, collision_count = 0;
      FOR_EACH_CANDIDATE(j, i, n, mode, &g, buf, cap, {
        const float *jp = pos_in + 2 * j;
        const float *jv = vel_in + 2 * j;
        if (dist2f(jp, ip) > interaction_radius) continue;
        gc[0] = gc[0] + jp[0];
        gc[1] = gc[1] + jp[1];
        gv[0] = gv[0] + jv[0];
        gv[1] = gv[1] + jv[1];
        interaction_count += 1;
        const float separation = dist2f(ip, jp);
        if (separation < separation_radius) {
          cc[0] = cc[0] + jp[0];
          cc[1] = cc[1] + jp[1];
          collision_count += 1;
        }
      });
      float vc[2] = {0, 0}, steer[2] = {0, 0}, match[2] = {0, 0}, avoid[2] = {0, 0};
      if (interaction_count > 0) {
        gc[0] = gc[0] / (float) interaction_count;
        gc[1] = gc[1] / (float) interaction_count;
        steer[0] = (gc[0] - ip[0]) * steer_scale;
        steer[1] = (gc[1] - ip[1]) * steer_scale;
      }
      vc[0] = vc[0] + steer[0];
      vc[1] = vc[1] + steer[1];
      if (interaction_count > 0) {
        gv[0] = gv[0] / (float) interaction_count;
        gv[1] = gv[1] / (float) interaction_count;
        match[0] = gv[0] * match_scale;
        match[1] = gv[1] * match_scale;
      }
      vc[0] = vc[0] + match[0];
      vc[1] = vc[1] + match[1];
      if (collision_count > 0) {
        cc[0] = cc[0] / (float) collision_count;
        cc[1] = cc[1] / (float) collision_count;
        avoid[0] = (ip[0] - cc[0]) * collision_scale;
        avoid[1] = (ip[1] - cc[1]) * collision_scale;
      }
      vc[0] = vc[0] + avoid[0];
      vc[1] = vc[1] + avoid[1];
      float nv[2] = {iv[0] + vc[0] * global_scale, iv[1] + vc[1] * global_scale};
      const float scale = sqrtf(nv[0] * nv[0] + nv[1] * nv[1]);
      if (scale > 1) {
        nv[0] = nv[0] / scale;
        nv[1] = nv[1] / scale;
      }
      for (int d = 0; d < 2; d++) {
        const float v = ip[d] + nv[d] * time_scale;
        pos_out[2 * i + d] = (v < min_pos) ? max_pos : ((v > max_pos) ? min_pos : v);
        vel_out[2 * i + d] = nv[d];
      }
    }
    free(buf);
  }
  if (mode == 1) {
    grid_free(&g);
    free(posd);
  }
  return 0;
}

/* ---------------------------------------------------- boids2d_flockers */
/* examples/boids2d_flockers.abl:39-86 as printed by the reference, run as
 * the reference program runs on one OpenMP thread: agents in index order,
 * each step's random(float2(-1.0), float2(1.0)) drawing from the one
 * xorshift stream (y first, as gcc on x86-64 evaluates
 * float2_create(random_float(..), random_float(..))).  Parameters:
 * p[0..8] = interaction_radius, steer_scale, collision_scale, match_scale,
 * randomness_scale, momentum_scale, time_scale, max_pos, (unused).
 * wraparound is asset/lib.abl's. */
ORACLE_API int oracle_flockers_step(long n, const double *pos_in, const double *vel_in,
                                    double *pos_out, double *vel_out, const double *p, int mode) {
  const double interaction_radius = p[0], steer_scale = p[1], collision_scale = p[2],
               match_scale = p[3], randomness_scale = p[4], momentum_scale = p[5],
               time_scale = p[6], max_pos = p[7];
  grid_t g;
  double emin[2] = {0, 0}, emax[2] = {max_pos, max_pos};
  if (mode == 1) grid_build(&g, 2, n, pos_in, emin, emax, interaction_radius);
  long *buf = NULL, cap = 0;
  for (long i = 0; i < n; i++) {
    const double *ip = pos_in + 2 * i;
    const double *iv = vel_in + 2 * i;
    double gv[2] = {0, 0}, gc[2] = {0, 0}, av[2] = {0, 0};
    int interaction_count = 0;
    FOR_EACH_CANDIDATE(j, i, n, mode, &g, buf, cap, {
      const double *jp = pos_in + 2 * j;
      const double *jv = vel_in + 2 * j;
      if (dist2(jp, ip) > interaction_radius) continue;
      if (jp[0] == ip[0] && jp[1] == ip[1]) continue;
      interaction_count += 1;
      gc[0] = gc[0] + jp[0];
      gc[1] = gc[1] + jp[1];
      gv[0] = gv[0] + jv[0];
      gv[1] = gv[1] + jv[1];
      const double sep[2] = {ip[0] - jp[0], ip[1] - jp[1]};
      const double lensquared = sep[0] * sep[0] + sep[1] * sep[1];
      const double den = lensquared * lensquared + 1;
      av[0] = av[0] + sep[0] / den;
      av[1] = av[1] + sep[1] / den;
    });
    double vc[2] = {0, 0};
    if (interaction_count > 0) {
      gc[0] = gc[0] / interaction_count;
      gc[1] = gc[1] / interaction_count;
      vc[0] = vc[0] + (gc[0] - ip[0]) * steer_scale;
      vc[1] = vc[1] + (gc[1] - ip[1]) * steer_scale;
      gv[0] = gv[0] / interaction_count;
      gv[1] = gv[1] / interaction_count;
      vc[0] = vc[0] + gv[0] * match_scale;
      vc[1] = vc[1] + gv[1] * match_scale;
      av[0] = av[0] / interaction_count;
      av[1] = av[1] / interaction_count;
      vc[0] = vc[0] + av[0] * collision_scale;
      vc[1] = vc[1] + av[1] * collision_scale;
    }
    double rd[2];
    const double lo[2] = {-1.0, -1.0}, hi[2] = {1.0, 1.0};
    draw_vec(rd, 2, lo, hi);
    const double rl = (double) sqrtf((float) (rd[0] * rd[0] + rd[1] * rd[1]));
    rd[0] = rd[0] / rl;
    rd[1] = rd[1] / rl;
    vc[0] = vc[0] + rd[0] * randomness_scale;
    vc[1] = vc[1] + rd[1] * randomness_scale;
    double nv[2] = {iv[0] * momentum_scale + vc[0], iv[1] * momentum_scale + vc[1]};
    const double scale = (double) sqrtf((float) (nv[0] * nv[0] + nv[1] * nv[1]));
    if (scale > 0) {
      nv[0] = nv[0] / scale;
      nv[1] = nv[1] / scale;
    }
    for (int d = 0; d < 2; d++) {
      const double v = ip[d] + nv[d] * time_scale;
      pos_out[2 * i + d] = (v < 0) ? (max_pos + v) : ((v >= max_pos) ? (v - max_pos) : v);
      vel_out[2 * i + d] = nv[d];
    }
  }
  free(buf);
  if (mode == 1) grid_free(&g);
  return 0;
}

/* ---------------------------------------------------------- sugarscape */
/* examples/sugarscape.abl:67-160, the four step functions as printed by the
 * reference.  Members of `out` a step does not write keep what the double
 * buffer held (agents_X_dbuf, src/backend/CPrinter.cpp:189-233: the dbuf
 * starts as a copy of the population and the two are swapped after every
 * step function), so `out` is passed in holding the double buffer and only
 * the members the printed code assigns are changed.  States: 0 unoccupied,
 * 1 occupied, 2 movement requested, 3 movement unresolved; the near radius is
 * the global `radius` and the sugar growback rate 1 (sugarscape.abl:28-39). */
typedef struct {
  double *pos, *target_pos;
  int *agent_id, *state, *sugar_level, *metabolism, *env_sugar_level, *max_env_sugar_level;
} sg_cols;

static inline int sg_same(const double *a, const double *b) { return a[0] == b[0] && a[1] == b[1]; }

ORACLE_API int oracle_sugarscape_step(int k, long n, const sg_cols *in, sg_cols *out,
                                      double radius, double grid_width, int mode, int nthreads) {
  enum { UNOCCUPIED = 0, OCCUPIED = 1, REQUESTED = 2, UNRESOLVED = 3 };
  grid_t g;
  double emin[2] = {0, 0}, emax[2] = {grid_width, grid_width};
  if (k > 0 && mode == 1) grid_build(&g, 2, n, in->pos, emin, emax, radius);
#pragma omp parallel num_threads(threads_or_default(nthreads))
  {
    long *buf = NULL, cap = 0;
#pragma omp for schedule(dynamic, 64)
    for (long i = 0; i < n; i++) {
      const double *ip = in->pos + 2 * i;
      if (k == 0) {
        /* metabolise_and_growback, sugarscape.abl:67-92 */
        int new_env = in->env_sugar_level[i];
        if (in->state[i] == OCCUPIED) {
          int new_sugar = in->sugar_level[i] + in->env_sugar_level[i] - in->metabolism[i];
          new_env = 0;
          if (new_sugar <= 0) {
            out->state[i] = UNOCCUPIED;
            out->agent_id[i] = -1;
            out->sugar_level[i] = 0;
            out->metabolism[i] = 0;
          } else {
            out->state[i] = UNRESOLVED;
            out->sugar_level[i] = new_sugar;
          }
        }
        new_env += 1;
        if (new_env > in->max_env_sugar_level[i]) new_env = in->max_env_sugar_level[i];
        out->env_sugar_level[i] = new_env;
      } else if (k == 1) {
        /* movement_request, sugarscape.abl:94-113: the first unoccupied
         * neighbour (ascending index) with the most sugar */
        if (in->state[i] != UNRESOLVED) continue;
        int best = -1;
        double best_pos[2] = {0, 0};
        FOR_EACH_CANDIDATE(j, i, n, mode, &g, buf, cap, {
          const double *jp = in->pos + 2 * j;
          if (dist2(jp, ip) > radius) continue;
          if (sg_same(jp, ip)) continue;
          if (in->state[j] == UNOCCUPIED && in->env_sugar_level[j] > best) {
            best = in->env_sugar_level[j];
            best_pos[0] = jp[0];
            best_pos[1] = jp[1];
          }
        });
        if (best > in->env_sugar_level[i]) {
          out->state[i] = REQUESTED;
          out->target_pos[2 * i] = best_pos[0];
          out->target_pos[2 * i + 1] = best_pos[1];
        } else {
          out->state[i] = OCCUPIED;
        }
      } else if (k == 2) {
        /* movement_response, sugarscape.abl:115-142: the first requester
         * (ascending index) whose target is this cell */
        if (in->state[i] != UNOCCUPIED) continue;
        int best_priority = -1, best_id = -1, best_sugar = -1, best_metab = -1;
        FOR_EACH_CANDIDATE(j, i, n, mode, &g, buf, cap, {
          const double *jp = in->pos + 2 * j;
          if (dist2(jp, ip) > radius) continue;
          if (in->state[j] == REQUESTED && sg_same(in->target_pos + 2 * j, ip)) {
            const int priority = 0;
            if (priority > best_priority) {
              best_priority = priority;
              best_id = in->agent_id[j];
              best_sugar = in->sugar_level[j];
              best_metab = in->metabolism[j];
            }
          }
        });
        if (best_id >= 0) {
          out->state[i] = OCCUPIED;
          out->agent_id[i] = best_id;
          out->sugar_level[i] = best_sugar;
          out->metabolism[i] = best_metab;
        }
      } else {
        /* movement_transaction, sugarscape.abl:144-160 */
        if (in->state[i] != REQUESTED) continue;
        int moved = 0;
        FOR_EACH_CANDIDATE(j, i, n, mode, &g, buf, cap, {
          const double *jp = in->pos + 2 * j;
          if (dist2(jp, ip) > radius) continue;
          if (in->state[j] == OCCUPIED && in->agent_id[j] == in->agent_id[i]) {
            moved = 1;
            out->state[i] = UNOCCUPIED;
            out->agent_id[i] = -1;
            out->sugar_level[i] = 0;
            out->metabolism[i] = 0;
          }
        });
        if (!moved) out->state[i] = OCCUPIED;
      }
    }
    free(buf);
  }
  if (k > 0 && mode == 1) grid_free(&g);
  return 0;
}

/* ------------------------------------------------------- predator_prey */
/* examples/predator_prey.abl:26-309.  The reference `c` backend refuses this
 * model (runtime add/remove, src/backend/CBackend.cpp:30-32), so its
 * semantics are stated here and followed by the CUDA path:
 *  - `out` starts as a copy of `in` (as the MASON backend's prepareOutState,
 *    src/backend/MasonPrinter.cpp:480-486);
 *  - after a step function, agents that called removeCurrent() are removed
 *    by a stable compaction, and agents created with add() are appended
 *    after the survivors in parent-index order;
 *  - random() in a step function draws from Philox4x32-10 (Salmon et al.,
 *    SC'11) with key (seed low, seed high) and counter (agent index, step
 *    function index in simulate order, timestep, draw number); a draw's 64
 *    bits (words 0 and 1) give u = (bits >> 11) * 2^-53 and
 *    random(lo, hi) = lo + u * (hi - lo), evaluated in abl_float (the one
 *    draw of the model, random(1.0), is therefore (abl_float) u);
 *  - the sequential step gather_stats runs after the parallel steps of every
 *    timestep (src/AnalysisVisitor.cpp:695-704).
 * Arithmetic follows the printed step bodies (float2 ops component-wise,
 * length = sqrtf of the float-rounded sum of squares). */

typedef struct {
  uint32_t k0, k1, c0, c1, c2, draw;
} pp_rng;

static void philox_next4(pp_rng *R, uint32_t out[4]) {
  uint32_t x0 = R->c0, x1 = R->c1, x2 = R->c2, x3 = R->draw++;
  uint32_t key0 = R->k0, key1 = R->k1;
  for (int r = 0; r < 10; r++) {
    if (r > 0) {
      key0 += 0x9E3779B9u;
      key1 += 0xBB67AE85u;
    }
    uint64_t p0 = (uint64_t) 0xD2511F53u * x0, p1 = (uint64_t) 0xCD9E8D57u * x2;
    uint32_t hi0 = (uint32_t) (p0 >> 32), lo0 = (uint32_t) p0;
    uint32_t hi1 = (uint32_t) (p1 >> 32), lo1 = (uint32_t) p1;
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

/* A draw's 53-bit uniform in [0, 1). */
static double pp_unit(pp_rng *R) {
  uint32_t x[4];
  philox_next4(R, x);
  uint64_t b = (((uint64_t) x[0] << 32) | x[1]) >> 11;
  return (double) b * (1.0 / 9007199254740992.0);
}

enum { PP_PRED = 0, PP_PREY = 1, PP_GRASS = 2 };

enum {
  S_PRED_FOLLOW_PREY, S_PREY_AVOID_PRED, S_PREY_FLOCK, S_PRED_AVOID, S_PREY_MOVE, S_PRED_MOVE,
  S_PREY_EAT_OR_STARVE, S_PRED_EAT_OR_STARVE, S_GRASS_EATEN, S_PREY_EATEN,
  S_PRED_REPRODUCTION, S_PREY_REPRODUCTION, S_GRASS_GROWTH, S_COUNT
};

static const int pp_step_type[S_COUNT] = {PP_PRED, PP_PREY, PP_PREY, PP_PRED, PP_PREY, PP_PRED,
                                         PP_PREY, PP_PRED, PP_GRASS, PP_PREY, PP_PRED, PP_PREY,
                                         PP_GRASS};

/* The FP64 build (oracle_pp_*) and the use_float build (oracle_pp_*_f32). */
#define PP_REAL double
#define PP_FN(x) x
#include "abl_oracle_pp.h"
#undef PP_REAL
#undef PP_FN
#define PP_REAL float
#define PP_FN(x) x##_f32
#include "abl_oracle_pp.h"
#undef PP_REAL
#undef PP_FN

/* ------------------------------------------------- device-side main() init */
/* examples/boids2d.abl:110-118 as `-b cuda -C cuda.device_init=true` runs it:
 * the loop `for (int i : 0..num_agents) add(Boid{pos: random(float2(min_pos),
 * float2(max_pos)), velocity: random(float2(-1), float2(1))})` becomes one
 * thread per iteration, drawing from the counter-based stream instead of the
 * reference's sequential xorshift stream.  The stated semantics:
 *  - iteration t of add() loop number L draws from Philox4x32-10 with key
 *    (0x5eed, 0) and counter (t, 0xffffff00 + L, 0, draw number);
 *  - random(float2 lo, float2 hi) draws y before x (the evaluation order the
 *    generator fixes for calls whose arguments draw, last argument first);
 *  - random(lo, hi) = lo + u * (hi - lo) with u the draw's 53-bit uniform. */
ORACLE_API void oracle_devinit_boids2d(long n, double min_pos, double max_pos, double *pos,
                                       double *vel) {
  for (long t = 0; t < n; t++) {
    pp_rng R;
    R.k0 = 0x5eedu;
    R.k1 = 0;
    R.c0 = (uint32_t) t;
    R.c1 = 0xffffff00u;
    R.c2 = 0;
    R.draw = 0;
    double py = min_pos + pp_unit(&R) * (max_pos - min_pos);
    double px = min_pos + pp_unit(&R) * (max_pos - min_pos);
    double vy = -1.0 + pp_unit(&R) * (1.0 - -1.0);
    double vx = -1.0 + pp_unit(&R) * (1.0 - -1.0);
    pos[2 * t] = px;
    pos[2 * t + 1] = py;
    vel[2 * t] = vx;
    vel[2 * t + 1] = vy;
  }
}
