/* predator_prey restatement, generic over the float width -- TEST
 * INFRASTRUCTURE ONLY, included by abl_oracle.c twice:
 *   PP_REAL double, PP_FN(x) x        the FP64 build (abl_float = double)
 *   PP_REAL float,  PP_FN(x) x##_f32  the use_float build (abl_float = float,
 *                                     asset/c/libabl.h:59-63)
 * The semantics are stated at the predator_prey section of abl_oracle.c.
 * Every member, printed constant and intermediate of the step bodies
 * (examples/predator_prey.abl:98-301) has type PP_REAL, as the printed C
 * declares them (`float2` and `float` are abl_float), and each operation is
 * evaluated in that type: float2 ops component-wise, length =
 * sqrtf((float) (x*x + y*y)), division by the int neighbour count after
 * converting it to PP_REAL.  Literals of the printed code (0.0, 1.0, -1.0)
 * are compared or multiplied where their value is exact in either width.
 * random(1.0) in a step is (PP_REAL) u with u the 53-bit Philox uniform.
 * Grid candidates are found from double copies of the positions (exact),
 * with the 1% cell margin; the in-radius test itself is the printed one. */

typedef struct {
  long n, cap;
  PP_REAL *pos, *dir, *steer; /* cap x 2 (dir/steer: animals only) */
  int *life;                  /* animals */
  int *dead_cycles;           /* grass */
  uint8_t *avail;             /* grass */
} PP_FN(pp_pop);

typedef struct {
  PP_FN(pp_pop) t[3];
  /* printed constants, stored as the program's globals are */
  PP_REAL PRED_PREY_INTERACTION_RADIUS, PREY_GROUP_COHESION_RADIUS,
      SAME_SPECIES_AVOIDANCE_RADIUS, GRASS_EAT_DISTANCE, PRED_KILL_DISTANCE, DELTA_TIME,
      PRED_SPEED_ADVANTAGE, SPACE_MULT, REPRODUCE_PREY_PROB, REPRODUCE_PREDATOR_PROB, env_size;
  int GAIN_FROM_FOOD_PREDATOR, GAIN_FROM_FOOD_PREY, GRASS_REGROW_CYCLES;
  uint64_t seed;
  long timestep;
} PP_FN(pp_sim);

static void PP_FN(pp_alloc)(PP_FN(pp_pop) *p, long cap, int grass) {
  p->cap = cap;
  p->pos = calloc(2 * cap, sizeof(PP_REAL));
  if (grass) {
    p->dead_cycles = calloc(cap, sizeof(int));
    p->avail = calloc(cap, 1);
  } else {
    p->dir = calloc(2 * cap, sizeof(PP_REAL));
    p->steer = calloc(2 * cap, sizeof(PP_REAL));
    p->life = calloc(cap, sizeof(int));
  }
}

static void PP_FN(pp_free)(PP_FN(pp_pop) *p) {
  free(p->pos);
  free(p->dir);
  free(p->steer);
  free(p->life);
  free(p->dead_cycles);
  free(p->avail);
  memset(p, 0, sizeof *p);
}

static void PP_FN(pp_copy_agent)(const PP_FN(pp_pop) *src, long i, PP_FN(pp_pop) *dst, long j,
                                 int grass) {
  dst->pos[2 * j] = src->pos[2 * i];
  dst->pos[2 * j + 1] = src->pos[2 * i + 1];
  if (grass) {
    dst->dead_cycles[j] = src->dead_cycles[i];
    dst->avail[j] = src->avail[i];
  } else {
    dst->dir[2 * j] = src->dir[2 * i];
    dst->dir[2 * j + 1] = src->dir[2 * i + 1];
    dst->steer[2 * j] = src->steer[2 * i];
    dst->steer[2 * j + 1] = src->steer[2 * i + 1];
    dst->life[j] = src->life[i];
  }
}

/* dparams: 11 printed constants (radii..env_size in the order of pp_sim),
 * rounded to PP_REAL as the program's globals are; iparams: 3 ints. */
ORACLE_API void *PP_FN(oracle_pp_create)(const double *dparams, const int *iparams,
                                         uint64_t seed, const long *n,
                                         const PP_REAL *const *pos, const PP_REAL *const *dir,
                                         const PP_REAL *const *steer, const int *const *life,
                                         const int *dead_cycles, const uint8_t *avail) {
  PP_FN(pp_sim) *S = calloc(1, sizeof *S);
  PP_REAL *d = &S->PRED_PREY_INTERACTION_RADIUS;
  for (int k = 0; k < 11; k++) d[k] = (PP_REAL) dparams[k];
  S->GAIN_FROM_FOOD_PREDATOR = iparams[0];
  S->GAIN_FROM_FOOD_PREY = iparams[1];
  S->GRASS_REGROW_CYCLES = iparams[2];
  S->seed = seed;
  for (int ti = 0; ti < 3; ti++) {
    long cap = 2 * n[ti] + 1024;
    PP_FN(pp_alloc)(&S->t[ti], cap, ti == PP_GRASS);
    S->t[ti].n = n[ti];
    memcpy(S->t[ti].pos, pos[ti], sizeof(PP_REAL) * 2 * n[ti]);
    if (ti == PP_GRASS) {
      memcpy(S->t[ti].dead_cycles, dead_cycles, sizeof(int) * n[ti]);
      memcpy(S->t[ti].avail, avail, n[ti]);
    } else {
      memcpy(S->t[ti].dir, dir[ti], sizeof(PP_REAL) * 2 * n[ti]);
      memcpy(S->t[ti].steer, steer[ti], sizeof(PP_REAL) * 2 * n[ti]);
      memcpy(S->t[ti].life, life[ti], sizeof(int) * n[ti]);
    }
  }
  return S;
}

ORACLE_API void PP_FN(oracle_pp_destroy)(void *h) {
  PP_FN(pp_sim) *S = h;
  for (int ti = 0; ti < 3; ti++) PP_FN(pp_free)(&S->t[ti]);
  free(S);
}

ORACLE_API long PP_FN(oracle_pp_count)(void *h, int type) {
  return ((PP_FN(pp_sim) *) h)->t[type].n;
}

ORACLE_API void PP_FN(oracle_pp_get)(void *h, int type, PP_REAL *pos, PP_REAL *dir,
                                     PP_REAL *steer, int *life, int *dead_cycles,
                                     uint8_t *avail) {
  PP_FN(pp_pop) *p = &((PP_FN(pp_sim) *) h)->t[type];
  memcpy(pos, p->pos, sizeof(PP_REAL) * 2 * p->n);
  if (type == PP_GRASS) {
    memcpy(dead_cycles, p->dead_cycles, sizeof(int) * p->n);
    memcpy(avail, p->avail, p->n);
  } else {
    memcpy(dir, p->dir, sizeof(PP_REAL) * 2 * p->n);
    memcpy(steer, p->steer, sizeof(PP_REAL) * 2 * p->n);
    memcpy(life, p->life, sizeof(int) * p->n);
  }
}

/* length_float2(float2_sub(a, b)) */
static inline PP_REAL PP_FN(len_sub)(const PP_REAL *a, const PP_REAL *b) {
  PP_REAL dx = a[0] - b[0], dy = a[1] - b[1];
  return (PP_REAL) sqrtf((float) (dx * dx + dy * dy));
}

static inline PP_REAL PP_FN(clampr)(PP_REAL v, PP_REAL lo, PP_REAL hi) {
  return (v < lo) ? lo : ((v > hi) ? hi : v);
}

/* Candidates of a near loop: all agents of `nb` (mode 0) or the sorted grid
 * candidates (mode 1), the in-radius test applied by the caller. */
typedef struct {
  int mode;
  grid_t g;
  const PP_FN(pp_pop) *nb;
} PP_FN(pp_near);

static void PP_FN(pp_near_init)(PP_FN(pp_near) *N, const PP_FN(pp_pop) *nb, double radius,
                                double env, int mode) {
  N->mode = mode;
  N->nb = nb;
  if (mode == 1) {
    double emin[2] = {0, 0}, emax[2] = {env, env};
    double *p = malloc(sizeof(double) * 2 * (nb->n ? nb->n : 1));
    for (long i = 0; i < 2 * nb->n; i++) p[i] = (double) nb->pos[i];
    grid_build(&N->g, 2, nb->n, p, emin, emax, radius);
    free(p);
  }
}

static void PP_FN(pp_near_free)(PP_FN(pp_near) *N) {
  if (N->mode == 1) grid_free(&N->g);
}

/* Candidate list of query position q (ascending neighbour index). */
static long PP_FN(pp_candidates)(const PP_FN(pp_near) *N, const PP_REAL *qr, long **buf,
                                 long *cap) {
  if (N->mode == 0) {
    if (N->nb->n > *cap) {
      *cap = N->nb->n + 64;
      *buf = realloc(*buf, *cap * sizeof(long));
    }
    for (long j = 0; j < N->nb->n; j++) (*buf)[j] = j;
    return N->nb->n;
  }
  const grid_t *g = &N->g;
  const double q[2] = {(double) qr[0], (double) qr[1]};
  long kx = (long) floor((q[0] - g->lo[0]) * g->inv_cell);
  long ky = (long) floor((q[1] - g->lo[1]) * g->inv_cell);
  kx = clampl(kx, 0, g->dims[0] - 1);
  ky = clampl(ky, 0, g->dims[1] - 1);
  long cnt = 0;
  for (long y = ky - 1; y <= ky + 1; y++) {
    if (y < 0 || y >= g->dims[1]) continue;
    for (long x = kx - 1; x <= kx + 1; x++) {
      if (x < 0 || x >= g->dims[0]) continue;
      long cc = y * g->dims[0] + x;
      long s = g->cell_start[cc], e = g->cell_start[cc + 1];
      if (cnt + (e - s) > *cap) {
        *cap = 2 * (cnt + (e - s)) + 64;
        *buf = realloc(*buf, *cap * sizeof(long));
      }
      for (long j = s; j < e; j++) (*buf)[cnt++] = g->order[j];
    }
  }
  qsort(*buf, cnt, sizeof(long), cmp_long);
  return cnt;
}

/* One step function over all agents of its type; `out` starts as `in`. */
static void PP_FN(pp_step)(PP_FN(pp_sim) *S, int k, int mode, int nthreads) {
  int ti = pp_step_type[k];
  PP_FN(pp_pop) *in = &S->t[ti];
  long n = in->n;
  int grass = ti == PP_GRASS;
  PP_FN(pp_pop) out;
  memset(&out, 0, sizeof out);
  PP_FN(pp_alloc)(&out, in->cap, grass);
  out.n = n;
  for (long i = 0; i < n; i++) PP_FN(pp_copy_agent)(in, i, &out, i, grass);
  uint8_t *removed = calloc(n ? n : 1, 1), *child = calloc(n ? n : 1, 1);
  PP_FN(pp_pop) kids;
  memset(&kids, 0, sizeof kids);
  PP_FN(pp_alloc)(&kids, n ? n : 1, grass);

  int near_type = -1;
  PP_REAL radius = 0;
  switch (k) {
    case S_PRED_FOLLOW_PREY: near_type = PP_PREY; radius = S->PRED_PREY_INTERACTION_RADIUS; break;
    case S_PREY_AVOID_PRED: near_type = PP_PRED; radius = S->PRED_PREY_INTERACTION_RADIUS; break;
    case S_PREY_FLOCK: near_type = PP_PREY; radius = S->PREY_GROUP_COHESION_RADIUS; break;
    case S_PRED_AVOID: near_type = PP_PRED; radius = S->SAME_SPECIES_AVOIDANCE_RADIUS; break;
    case S_PREY_EAT_OR_STARVE: near_type = PP_GRASS; radius = S->GRASS_EAT_DISTANCE; break;
    case S_PRED_EAT_OR_STARVE: near_type = PP_PREY; radius = S->PRED_KILL_DISTANCE; break;
    case S_GRASS_EATEN: near_type = PP_PREY; radius = S->GRASS_EAT_DISTANCE; break;
    case S_PREY_EATEN: near_type = PP_PRED; radius = S->PRED_KILL_DISTANCE; break;
    default: break;
  }
  PP_FN(pp_near) N;
  memset(&N, 0, sizeof N);
  if (near_type >= 0)
    PP_FN(pp_near_init)(&N, &S->t[near_type], (double) radius, (double) S->env_size, mode);
  const PP_FN(pp_pop) *nb = near_type >= 0 ? &S->t[near_type] : NULL;

/* The printed near loop: candidates in ascending index, skipped when
 * dist(nx.pos, in.pos) > radius (src/backend/CPrinter.cpp:160-170). */
#define PP_NEAR_LOOP(q, j, ...)                                                   \
  do {                                                                            \
    long cnt_ = PP_FN(pp_candidates)(&N, (q), &buf, &bcap);                       \
    for (long q_ = 0; q_ < cnt_; q_++) {                                          \
      long j = buf[q_];                                                           \
      if (PP_FN(len_sub)(nb->pos + 2 * j, (q)) > radius) continue;                \
      __VA_ARGS__                                                                 \
    }                                                                             \
  } while (0)

#pragma omp parallel num_threads(threads_or_default(nthreads))
  {
    long *buf = NULL, bcap = 0;
#pragma omp for schedule(dynamic, 256)
    for (long i = 0; i < n; i++) {
      const PP_REAL *ip = in->pos + 2 * i;
      switch (k) {
        case S_PRED_FOLLOW_PREY: {
          PP_REAL steer[2] = {0, 0}, cpp[2] = {0, 0};
          PP_REAL cpd = S->PRED_PREY_INTERACTION_RADIUS;
          int see = 0;
          PP_NEAR_LOOP(ip, j, {
            const PP_REAL *jp = nb->pos + 2 * j;
            PP_REAL sep = PP_FN(len_sub)(ip, jp);
            if (sep < cpd) {
              cpp[0] = jp[0];
              cpp[1] = jp[1];
              cpd = sep;
              see = 1;
            }
          });
          if (see) {
            steer[0] = cpp[0] - ip[0];
            steer[1] = cpp[1] - ip[1];
          }
          out.steer[2 * i] = steer[0];
          out.steer[2 * i + 1] = steer[1];
          break;
        }
        case S_PREY_AVOID_PRED:
        case S_PRED_AVOID: {
          PP_REAL R = k == S_PREY_AVOID_PRED ? S->PRED_PREY_INTERACTION_RADIUS
                                             : S->SAME_SPECIES_AVOIDANCE_RADIUS;
          PP_REAL av[2] = {0, 0};
          PP_NEAR_LOOP(ip, j, {
            const PP_REAL *jp = nb->pos + 2 * j;
            PP_REAL sep = PP_FN(len_sub)(ip, jp);
            int cond = k == S_PREY_AVOID_PRED
                           ? sep < R
                           : ((sep < R) && (jp[0] != ip[0] || jp[1] != ip[1]));
            if (cond && sep > 0.0) {
              PP_REAL s = R / sep;
              av[0] = av[0] + (ip[0] - jp[0]) * s;
              av[1] = av[1] + (ip[1] - jp[1]) * s;
            }
          });
          if (k == S_PREY_AVOID_PRED) {
            out.steer[2 * i] = av[0];
            out.steer[2 * i + 1] = av[1];
          } else {
            out.steer[2 * i] = in->steer[2 * i] + av[0];
            out.steer[2 * i + 1] = in->steer[2 * i + 1] + av[1];
          }
          break;
        }
        case S_PREY_FLOCK: {
          PP_REAL gc[2] = {0, 0}, gv[2] = {0, 0}, av[2] = {0, 0};
          int cnt = 0;
          PP_REAL R = S->SAME_SPECIES_AVOIDANCE_RADIUS;
          PP_NEAR_LOOP(ip, j, {
            const PP_REAL *jp = nb->pos + 2 * j;
            PP_REAL sep = PP_FN(len_sub)(ip, jp);
            gc[0] = gc[0] + jp[0];
            gc[1] = gc[1] + jp[1];
            cnt += 1;
            if ((sep < R) && (jp[0] != ip[0] || jp[1] != ip[1])) {
              if (sep > 0.0) {
                PP_REAL s = R / sep;
                av[0] = av[0] + (ip[0] - jp[0]) * s;
                av[1] = av[1] + (ip[1] - jp[1]) * s;
              }
            }
          });
          if (cnt > 0) {
            gc[0] = gc[0] / (PP_REAL) cnt;
            gc[1] = gc[1] / (PP_REAL) cnt;
            gv[0] = gc[0] - ip[0];
            gv[1] = gc[1] - ip[1];
          }
          out.steer[2 * i] = (in->steer[2 * i] + gv[0]) + av[0];
          out.steer[2 * i + 1] = (in->steer[2 * i + 1] + gv[1]) + av[1];
          break;
        }
        case S_PREY_MOVE:
        case S_PRED_MOVE: {
          PP_REAL p[2] = {ip[0], ip[1]};
          PP_REAL v[2] = {in->dir[2 * i] + in->steer[2 * i],
                          in->dir[2 * i + 1] + in->steer[2 * i + 1]};
          PP_REAL cs = (PP_REAL) sqrtf((float) (v[0] * v[0] + v[1] * v[1]));
          if (cs > 1.0) {
            PP_REAL l = (PP_REAL) sqrtf((float) (v[0] * v[0] + v[1] * v[1]));
            v[0] = v[0] / l;
            v[1] = v[1] / l;
          }
          for (int d = 0; d < 2; d++) {
            PP_REAL step = k == S_PREY_MOVE
                               ? (v[d] * S->DELTA_TIME) * S->SPACE_MULT
                               : ((v[d] * S->DELTA_TIME) * S->PRED_SPEED_ADVANTAGE)
                                     * S->SPACE_MULT;
            p[d] = p[d] + step;
            /* boundPosition -> clamp(pos, float2(env_size)) */
            p[d] = PP_FN(clampr)(p[d], (PP_REAL) 0, S->env_size);
          }
          out.pos[2 * i] = p[0];
          out.pos[2 * i + 1] = p[1];
          out.dir[2 * i] = v[0];
          out.dir[2 * i + 1] = v[1];
          out.life[i] = in->life[i] - 1;
          break;
        }
        case S_PREY_EAT_OR_STARVE:
        case S_PRED_EAT_OR_STARVE: {
          int life = in->life[i];
          PP_NEAR_LOOP(ip, j, {
            if (k == S_PREY_EAT_OR_STARVE) {
              if (nb->avail[j]) life += S->GAIN_FROM_FOOD_PREY;
            } else {
              life += S->GAIN_FROM_FOOD_PREDATOR;
            }
          });
          out.life[i] = life;
          if (life < 1) removed[i] = 1;
          break;
        }
        case S_GRASS_EATEN:
        case S_PREY_EATEN: {
          PP_REAL closest = k == S_GRASS_EATEN ? S->GRASS_EAT_DISTANCE : S->PRED_KILL_DISTANCE;
          int eaten = 0;
          PP_NEAR_LOOP(ip, j, {
            const PP_REAL *jp = nb->pos + 2 * j;
            if (k == S_GRASS_EATEN) {
              PP_REAL distance = PP_FN(len_sub)(ip, jp);
              if ((distance < closest) && in->avail[i]) {
                closest = distance;
                eaten = 1;
              }
            } else {
              PP_REAL distance = PP_FN(len_sub)(jp, ip);
              if (distance < closest) {
                closest = distance;
                eaten = 1;
              }
            }
          });
          if (k == S_GRASS_EATEN) {
            if (eaten) {
              out.dead_cycles[i] = 0;
              out.avail[i] = 0;
            }
          } else if (eaten) {
            removed[i] = 1;
          }
          break;
        }
        case S_PRED_REPRODUCTION:
        case S_PREY_REPRODUCTION: {
          pp_rng R;
          R.k0 = (uint32_t) S->seed;
          R.k1 = (uint32_t) (S->seed >> 32);
          R.c0 = (uint32_t) i;
          R.c1 = (uint32_t) k;
          R.c2 = (uint32_t) S->timestep;
          R.draw = 0;
          PP_REAL prob = k == S_PREY_REPRODUCTION ? S->REPRODUCE_PREY_PROB
                                                  : S->REPRODUCE_PREDATOR_PROB;
          /* random(1.0) = 0 + u * (1 - 0) in PP_REAL */
          if ((PP_REAL) pp_unit(&R) < prob) {
            child[i] = 1;
            kids.pos[2 * i] = ip[0];
            kids.pos[2 * i + 1] = ip[1];
            kids.dir[2 * i] = in->dir[2 * i] * (PP_REAL) -1.0;
            kids.dir[2 * i + 1] = in->dir[2 * i + 1] * (PP_REAL) -1.0;
            kids.steer[2 * i] = in->steer[2 * i] * (PP_REAL) -1.0;
            kids.steer[2 * i + 1] = in->steer[2 * i + 1] * (PP_REAL) -1.0;
            kids.life[i] = in->life[i] / 2;
            out.life[i] = in->life[i] / 2;
          }
          break;
        }
        case S_GRASS_GROWTH: {
          if (in->dead_cycles[i] == S->GRASS_REGROW_CYCLES) {
            out.dead_cycles[i] = 0;
            out.avail[i] = 1;
          }
          if (!in->avail[i]) out.dead_cycles[i] = in->dead_cycles[i] + 1;
          break;
        }
      }
    }
    free(buf);
  }
#undef PP_NEAR_LOOP
  if (near_type >= 0) PP_FN(pp_near_free)(&N);

  /* Survivors (stable) then children in parent order. */
  long survivors = 0, kids_n = 0;
  for (long i = 0; i < n; i++) {
    survivors += !removed[i];
    kids_n += child[i];
  }
  long need = survivors + kids_n;
  PP_FN(pp_pop) res;
  memset(&res, 0, sizeof res);
  long cap = in->cap > need ? in->cap : 2 * need + 1024;
  PP_FN(pp_alloc)(&res, cap, grass);
  long j = 0;
  for (long i = 0; i < n; i++)
    if (!removed[i]) PP_FN(pp_copy_agent)(&out, i, &res, j++, grass);
  for (long i = 0; i < n; i++)
    if (child[i]) PP_FN(pp_copy_agent)(&kids, i, &res, j++, grass);
  res.n = need;
  PP_FN(pp_free)(in);
  *in = res;
  PP_FN(pp_free)(&out);
  PP_FN(pp_free)(&kids);
  free(removed);
  free(child);
}

/* Runs `timesteps` timesteps; stats (3 ints per timestep: count(Prey),
 * count(Predator), sum(Grass.avail)) are written to `stats` if not NULL. */
ORACLE_API void PP_FN(oracle_pp_run)(void *h, int timesteps, int mode, int nthreads,
                                     int *stats) {
  PP_FN(pp_sim) *S = h;
  for (int t = 0; t < timesteps; t++) {
    for (int k = 0; k < S_COUNT; k++) PP_FN(pp_step)(S, k, mode, nthreads);
    S->timestep++;
    if (stats) {
      long g = 0;
      for (long i = 0; i < S->t[PP_GRASS].n; i++) g += S->t[PP_GRASS].avail[i];
      stats[3 * t] = (int) S->t[PP_PREY].n;
      stats[3 * t + 1] = (int) S->t[PP_PRED].n;
      stats[3 * t + 2] = (int) g;
    }
  }
}
