// Generated by OpenABL -b cuda (model "predator_prey").
#include "abl_gen.cuh"

namespace abl_model_predator_prey {

typedef double abl_float;
#include "abl_math.cuh"

typedef struct {
    float2 pos;
    float2 dir;
    float2 steer;
    int life;
} Predator;
static const type_info Predator_info[] = {
    { TYPE_FLOAT2, offsetof(Predator, pos), "pos", true },
    { TYPE_FLOAT2, offsetof(Predator, dir), "dir", false },
    { TYPE_FLOAT2, offsetof(Predator, steer), "steer", false },
    { TYPE_INT, offsetof(Predator, life), "life", false },
    { TYPE_END, sizeof(Predator), NULL }
};

typedef struct {
    float2 pos;
    float2 dir;
    float2 steer;
    int life;
} Prey;
static const type_info Prey_info[] = {
    { TYPE_FLOAT2, offsetof(Prey, pos), "pos", true },
    { TYPE_FLOAT2, offsetof(Prey, dir), "dir", false },
    { TYPE_FLOAT2, offsetof(Prey, steer), "steer", false },
    { TYPE_INT, offsetof(Prey, life), "life", false },
    { TYPE_END, sizeof(Prey), NULL }
};

typedef struct {
    float2 pos;
    int dead_cycles;
    bool avail;
} Grass;
static const type_info Grass_info[] = {
    { TYPE_FLOAT2, offsetof(Grass, pos), "pos", true },
    { TYPE_INT, offsetof(Grass, dead_cycles), "dead_cycles", false },
    { TYPE_BOOL, offsetof(Grass, avail), "avail", false },
    { TYPE_END, sizeof(Grass), NULL }
};

struct agent_struct {
    dyn_array agents_Predator;
    dyn_array agents_Predator_dbuf;
    dyn_array agents_Prey;
    dyn_array agents_Prey_dbuf;
    dyn_array agents_Grass;
    dyn_array agents_Grass_dbuf;
};
static struct agent_struct agents;
static const agent_info agents_info[] = {
    { Predator_info, offsetof(struct agent_struct, agents_Predator), "Predator" },
    { Prey_info, offsetof(struct agent_struct, agents_Prey), "Prey" },
    { Grass_info, offsetof(struct agent_struct, agents_Grass), "Grass" },
    { NULL, 0, NULL }
};

struct abl_globals {
    double PI;
    double SPACE_MULT;
    double REPRODUCE_PREY_PROB;
    double REPRODUCE_PREDATOR_PROB;
    int GAIN_FROM_FOOD_PREDATOR;
    int GAIN_FROM_FOOD_PREY;
    int GRASS_REGROW_CYCLES;
    double PRED_PREY_INTERACTION_RADIUS;
    double PREY_GROUP_COHESION_RADIUS;
    double SAME_SPECIES_AVOIDANCE_RADIUS;
    double GRASS_EAT_DISTANCE;
    double PRED_KILL_DISTANCE;
    double DELTA_TIME;
    double PRED_SPEED_ADVANTAGE;
    double prey_fraction;
    double predator_fraction;
    double agent_density;
    int num_agents;
    int num_timesteps;
    double env_size;
};
static const abl_globals abl_globals_default = {
    3.14159,
    1.0,
    0.005,
    0.001,
    35,
    60,
    60,
    0.1,
    0.12,
    0.035,
    0.02,
    0.02,
    0.0015,
    2.0,
    0.35,
    0.025,
    1600.0,
    3200,
    100,
    1.41421,
};
static abl_globals abl_G = abl_globals_default;
static abl::rng abl_R;  // unused on the host: main() draws from the host stream
struct abl_cols_Predator {
    float2 *pos;
    float2 *dir;
    float2 *steer;
    int *life;
};
struct abl_cols_Prey {
    float2 *pos;
    float2 *dir;
    float2 *steer;
    int *life;
};
struct abl_cols_Grass {
    float2 *pos;
    int *dead_cycles;
    bool *avail;
};
__device__ static void abl_add_Predator(abl::step_ctx &K, const Predator &c) {
    K.added = 1;
    ((float2 *) K.child_cols[0])[K.self] = c.pos;
    ((float2 *) K.child_cols[1])[K.self] = c.dir;
    ((float2 *) K.child_cols[2])[K.self] = c.steer;
    ((int *) K.child_cols[3])[K.self] = c.life;
}
__device__ static void abl_add_Prey(abl::step_ctx &K, const Prey &c) {
    K.added = 1;
    ((float2 *) K.child_cols[0])[K.self] = c.pos;
    ((float2 *) K.child_cols[1])[K.self] = c.dir;
    ((float2 *) K.child_cols[2])[K.self] = c.steer;
    ((int *) K.child_cols[3])[K.self] = c.life;
}
__device__ static void abl_add_Grass(abl::step_ctx &K, const Grass &c) {
    K.added = 1;
    ((float2 *) K.child_cols[0])[K.self] = c.pos;
    ((int *) K.child_cols[1])[K.self] = c.dead_cycles;
    ((bool *) K.child_cols[2])[K.self] = c.avail;
}

__host__ __device__ static inline float2 random_1(const abl_globals &abl_G, abl::rng &abl_R, float2 min, float2 max) {
    return ([&]() { const auto abl_e1_1 = abl_random(abl_R, min.y, max.y); const auto abl_e1_0 = abl_random(abl_R, min.x, max.x); return float2_create(abl_e1_0, abl_e1_1); }());
}
__host__ __device__ static inline float3 random_2(const abl_globals &abl_G, abl::rng &abl_R, float3 min, float3 max) {
    return ([&]() { const auto abl_e2_2 = abl_random(abl_R, min.z, max.z); const auto abl_e2_1 = abl_random(abl_R, min.y, max.y); const auto abl_e2_0 = abl_random(abl_R, min.x, max.x); return float3_create(abl_e2_0, abl_e2_1, abl_e2_2); }());
}
__host__ __device__ static inline double random_3(const abl_globals &abl_G, abl::rng &abl_R, double max) {
    return abl_random(abl_R, 0, max);
}
__host__ __device__ static inline float2 random_4(const abl_globals &abl_G, abl::rng &abl_R, float2 max) {
    return random_1(abl_G, abl_R, float2_fill(0), max);
}
__host__ __device__ static inline float3 random_5(const abl_globals &abl_G, abl::rng &abl_R, float3 max) {
    return random_2(abl_G, abl_R, float3_fill(0), max);
}
__host__ __device__ static inline int randomInt_1(const abl_globals &abl_G, abl::rng &abl_R, int max) {
    return abl_random_int(abl_R, 0, max);
}
__host__ __device__ static inline double clamp(const abl_globals &abl_G, abl::rng &abl_R, double pos, double min, double max) {
    return ((pos < min) ? min : ((pos > max) ? max : pos));
}
__host__ __device__ static inline float2 clamp_1(const abl_globals &abl_G, abl::rng &abl_R, float2 pos, float2 min, float2 max) {
    return float2_create(((pos.x < min.x) ? min.x : ((pos.x > max.x) ? max.x : pos.x)), ((pos.y < min.y) ? min.y : ((pos.y > max.y) ? max.y : pos.y)));
}
__host__ __device__ static inline float3 clamp_2(const abl_globals &abl_G, abl::rng &abl_R, float3 pos, float3 min, float3 max) {
    return float3_create(((pos.x < min.x) ? min.x : ((pos.x > max.x) ? max.x : pos.x)), ((pos.y < min.y) ? min.y : ((pos.y > max.y) ? max.y : pos.y)), ((pos.z < min.z) ? min.z : ((pos.z > max.z) ? max.z : pos.z)));
}
__host__ __device__ static inline double clamp_3(const abl_globals &abl_G, abl::rng &abl_R, double pos, double max) {
    return clamp(abl_G, abl_R, pos, 0, max);
}
__host__ __device__ static inline float2 clamp_4(const abl_globals &abl_G, abl::rng &abl_R, float2 pos, float2 max) {
    return clamp_1(abl_G, abl_R, pos, float2_fill(0), max);
}
__host__ __device__ static inline float3 clamp_5(const abl_globals &abl_G, abl::rng &abl_R, float3 pos, float3 max) {
    return clamp_2(abl_G, abl_R, pos, float3_fill(0), max);
}
__host__ __device__ static inline double wraparound(const abl_globals &abl_G, abl::rng &abl_R, double pos, double max) {
    return ((pos < 0) ? (max + pos) : ((pos >= max) ? (pos - max) : pos));
}
__host__ __device__ static inline float2 wraparound_1(const abl_globals &abl_G, abl::rng &abl_R, float2 pos, float2 max) {
    return float2_create(((pos.x < 0) ? (max.x + pos.x) : ((pos.x >= max.x) ? (pos.x - max.x) : pos.x)), ((pos.y < 0) ? (max.y + pos.y) : ((pos.y >= max.y) ? (pos.y - max.y) : pos.y)));
}
__host__ __device__ static inline float3 wraparound_2(const abl_globals &abl_G, abl::rng &abl_R, float3 pos, float3 max) {
    return float3_create(((pos.x < 0) ? (max.x + pos.x) : ((pos.x >= max.x) ? (pos.x - max.x) : pos.x)), ((pos.y < 0) ? (max.y + pos.y) : ((pos.y >= max.y) ? (pos.y - max.y) : pos.y)), ((pos.z < 0) ? (max.z + pos.z) : ((pos.z >= max.z) ? (pos.z - max.z) : pos.z)));
}
__host__ __device__ static inline bool is_inside(const abl_globals &abl_G, abl::rng &abl_R, float2 pos, float2 max) {
    return ((((pos.x >= 0) && (pos.y >= 0)) && (pos.x <= max.x)) && (pos.y <= max.y));
}
__host__ __device__ static inline float2 randomDirection(const abl_globals &abl_G, abl::rng &abl_R) {
    double phi = random_3(abl_G, abl_R, (2.0 * abl_G.PI));
    return float2_create(sin(phi), cos(phi));
}
__host__ __device__ static inline float2 boundPosition(const abl_globals &abl_G, abl::rng &abl_R, float2 pos) {
    return clamp_4(abl_G, abl_R, pos, float2_create(abl_G.env_size, abl_G.env_size));
}
__device__ static void prey_avoid_pred(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Prey* in, Prey* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    float2 avoid_velocity = float2_fill(0.0);
    {
        const abl::near_query<2> abl_q1(abl_NB, (double) in->pos.x, (double) in->pos.y, 0.0, abl_K.self);
        abl::near_list_cursor<2> abl_c1(abl_NB, abl_q1, abl_K);
        auto abl_exact1 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) abl_NB.cols[0])[abl_s];
            return !(dist_float2(abl_p, in->pos) > abl_G.PRED_PREY_INTERACTION_RADIUS);
        };
        while (abl_c1.fill(abl_q1, abl_exact1)) {
            int abl_pslot1 = abl_c1.slot(0);
            Predator abl_pnx1;
            abl_pnx1.pos = ((const float2 *) abl_NB.cols[0])[abl_pslot1];
            unsigned long long abl_dm1_0 = 0ull;
            for (int abl_k = 0; abl_k < abl_c1.cnt; ++abl_k) {
                const int abl_slot1 = abl_pslot1;
                Predator abl_nx1 = abl_pnx1;
                if (abl_k + 1 < abl_c1.cnt) {
                    abl_pslot1 = abl_c1.slot(abl_k + 1);
                    abl_pnx1.pos = ((const float2 *) abl_NB.cols[0])[abl_pslot1];
                }
                Predator* pred = &abl_nx1;
                {
                    const auto separation = abl::make_lazy_dist(abl_q1, abl_NB, abl_slot1, [&]() -> abl_float { return length_float2(float2_sub(in->pos, pred->pos)); });
                    if ((separation < abl_G.PRED_PREY_INTERACTION_RADIUS)) abl_dm1_0 |= 1ull << abl_k;
                }
            }
            for (unsigned long long abl_m = abl_dm1_0; abl_m; abl_m &= abl_m - 1ull) {
                const int abl_slot1 = abl_c1.slot(__ffsll((long long) abl_m) - 1);
                Predator abl_nx1;
                abl_nx1.pos = ((const float2 *) abl_NB.cols[0])[abl_slot1];
                Predator* pred = &abl_nx1;
                double separation = length_float2(float2_sub(in->pos, pred->pos));
                {
                    if ((separation > 0.0)) {
                        avoid_velocity = float2_add(avoid_velocity, float2_mul_scalar(float2_sub(in->pos, pred->pos), (abl_G.PRED_PREY_INTERACTION_RADIUS / separation)));
                    }
                }
            }
        }
    }
    out->steer = avoid_velocity;
}

#ifndef ABL_PERSIST
struct abl_kargs_prey_avoid_pred {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Prey in, out;
    abl_near_view NB;
    uint8_t *removed;
    uint8_t *child_flag;
    void *child_cols[ABL_MAX_MEMBERS];
    uint64_t seed;
    long timestep;
    int step_index;
    uint32_t skip_store;
    unsigned long long *serial_rng;
};
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_prey_avoid_pred(const __grid_constant__ abl_kargs_prey_avoid_pred A) {
    int abl_j;
    {
        const abl_globals &abl_G = A.G;
        const long abl_t1 = (long) blockIdx.x * blockDim.x + threadIdx.x;
        const bool abl_has = abl_t1 < A.n;
        const long abl_i1 = abl_has ? (A.visit ? (long) A.visit[abl_t1] : abl_t1) : 0;
        const float2 abl_p1 = abl_has ? A.in.pos[abl_i1] : float2{};
        const abl::near_query<2> abl_q0(A.NB, (double) abl_p1.x, (double) abl_p1.y, 0.0, abl_has ? abl_i1 : -1);
        auto abl_x0 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) A.NB.cols[0])[abl_s];
            return !(dist_float2(abl_p, abl_p1) > abl_G.PRED_PREY_INTERACTION_RADIUS);
        };
        abl_j = abl::presort_block<2>(A.NB, abl_has, abl_q0, abl_x0);
    }
    const long abl_t = (long) blockIdx.x * blockDim.x + abl_j;
    if (abl_t >= A.n) return;
    const long abl_i = A.visit ? (long) A.visit[abl_t] : abl_t;
    abl::step_ctx abl_K;
    abl_K.R.init(A.seed, (uint32_t) abl_i, (uint32_t) A.step_index, (uint64_t) A.timestep);
    abl_K.R.xs = A.serial_rng;
    abl_K.self = abl_i;
    abl_K.removed = 0;
    abl_K.added = 0;
    abl_K.child_cols = A.child_cols;
    abl_K.near_col = abl_j;
    Prey abl_in, abl_out;
    abl_in.pos = A.in.pos[abl_i];
    abl_in.dir = A.in.dir[abl_i];
    abl_in.steer = A.in.steer[abl_i];
    abl_in.life = A.in.life[abl_i];
    abl_out = abl_in;
    prey_avoid_pred(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.pos[abl_i] = abl_out.pos;
    A.out.dir[abl_i] = abl_out.dir;
    A.out.steer[abl_i] = abl_out.steer;
    A.out.life[abl_i] = abl_out.life;
}
static int abl_launch_prey_avoid_pred(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_prey_avoid_pred A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.pos = (float2 *) L->in_cols[0];
    A.out.pos = (float2 *) L->out_cols[0];
    A.in.dir = (float2 *) L->in_cols[1];
    A.out.dir = (float2 *) L->out_cols[1];
    A.in.steer = (float2 *) L->in_cols[2];
    A.out.steer = (float2 *) L->out_cols[2];
    A.in.life = (int *) L->in_cols[3];
    A.out.life = (int *) L->out_cols[3];
    A.NB = L->near;
    A.removed = L->removed;
    A.child_flag = L->child_flag;
    for (int k = 0; k < ABL_MAX_MEMBERS; k++) A.child_cols[k] = L->child_cols[k];
    A.seed = L->seed;
    A.timestep = L->timestep;
    A.step_index = L->step_index;
    A.skip_store = L->skip_store;
    A.serial_rng = L->serial_rng;
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (A.n + abl_block - 1) / abl_block;
    abl_kernel_prey_avoid_pred<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
__device__ __forceinline__ void abl_ens_body_prey_avoid_pred(const abl_ens_launch &A, long abl_vb, long abl_ts) {
    int abl_j;
    {
        const long abl_t1 = abl_vb * blockDim.x + threadIdx.x;
        const bool abl_has = abl_t1 < A.n;
        const long abl_i1 = abl_has ? (A.visit_order ? (long) A.visit_order[abl_t1] : abl_t1) : 0;
        const int abl_r1 = abl_has ? A.replica[abl_i1] : 0;
        const abl_globals &abl_G = ((const abl_globals *) A.globals)[abl_r1];
        const abl_near_view &abl_V1 = A.views[abl_r1];
        const float2 abl_p1 = abl_has ? ((const float2 *) A.in_cols[0])[abl_i1] : float2{};
        const abl::near_query<2> abl_q0(abl_V1, (double) abl_p1.x, (double) abl_p1.y, 0.0, abl_has ? abl_i1 : -1);
        auto abl_x0 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) abl_V1.cols[0])[abl_s];
            return !(dist_float2(abl_p, abl_p1) > abl_G.PRED_PREY_INTERACTION_RADIUS);
        };
        abl_j = abl::presort_block<2>(abl_V1, abl_has, abl_q0, abl_x0);
    }
    const long abl_t = abl_vb * blockDim.x + abl_j;
    if (abl_t >= A.n) return;
    const long abl_i = A.visit_order ? (long) A.visit_order[abl_t] : abl_t;
    const int abl_r = A.replica[abl_i];
    const abl_globals &abl_Gr = ((const abl_globals *) A.globals)[abl_r];
    abl::step_ctx abl_K;
    abl_K.R.init(A.seeds[abl_r], (uint32_t) (abl_i - A.agent_base[abl_r]), (uint32_t) A.step_index, (uint64_t) abl_ts);
    abl_K.self = abl_i;
    abl_K.removed = 0;
    abl_K.added = 0;
    abl_K.child_cols = nullptr;
    abl_K.near_col = abl_j;
    Prey abl_in, abl_out;
    abl_in.pos = ((const float2 *) A.in_cols[0])[abl_i];
    abl_in.dir = ((const float2 *) A.in_cols[1])[abl_i];
    abl_in.steer = ((const float2 *) A.in_cols[2])[abl_i];
    abl_in.life = ((const int *) A.in_cols[3])[abl_i];
    abl_out.pos = abl_in.pos;
    abl_out.dir = abl_in.dir;
    abl_out.steer = abl_in.steer;
    abl_out.life = abl_in.life;
    prey_avoid_pred(abl_Gr, A.views[abl_r], abl_K, &abl_in, &abl_out);
    ((float2 *) A.out_cols[0])[abl_i] = abl_out.pos;
    ((float2 *) A.out_cols[1])[abl_i] = abl_out.dir;
    ((float2 *) A.out_cols[2])[abl_i] = abl_out.steer;
    ((int *) A.out_cols[3])[abl_i] = abl_out.life;
}
#ifndef ABL_PERSIST
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ens_prey_avoid_pred(const __grid_constant__ abl_ens_launch A) {
    abl_ens_body_prey_avoid_pred(A, blockIdx.x, A.timestep);
}
static int abl_launch_ens_prey_avoid_pred(const abl_ens_launch *L, cudaStream_t abl_stream) {
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (L->n + abl_block - 1) / abl_block;
    abl_kernel_ens_prey_avoid_pred<<<abl_grid, abl_block, L->smem, abl_stream>>>(*L);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
#ifndef ABL_PERSIST
static double abl_radius_prey_avoid_pred(const void *abl_gp) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    return (double) (abl_G.PRED_PREY_INTERACTION_RADIUS);
}
#endif

__device__ static void prey_flock(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Prey* in, Prey* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    float2 group_center = float2_fill(0.0);
    float2 group_velocity = float2_fill(0.0);
    float2 avoid_velocity = float2_fill(0.0);
    int group_centre_count = 0;
    {
        const abl::near_query<2> abl_q2(abl_NB, (double) in->pos.x, (double) in->pos.y, 0.0, abl_K.self);
        abl::near_list_cursor<2> abl_c2(abl_NB, abl_q2, abl_K);
        auto abl_exact2 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) abl_NB.cols[0])[abl_s];
            return !(dist_float2(abl_p, in->pos) > abl_G.PREY_GROUP_COHESION_RADIUS);
        };
        while (abl_c2.fill(abl_q2, abl_exact2)) {
            int abl_pslot2 = abl_c2.slot(0);
            Prey abl_pnx2;
            abl_pnx2.pos = ((const float2 *) abl_NB.cols[0])[abl_pslot2];
            unsigned long long abl_dm2_0 = 0ull;
            for (int abl_k = 0; abl_k < abl_c2.cnt; ++abl_k) {
                const int abl_slot2 = abl_pslot2;
                Prey abl_nx2 = abl_pnx2;
                if (abl_k + 1 < abl_c2.cnt) {
                    abl_pslot2 = abl_c2.slot(abl_k + 1);
                    abl_pnx2.pos = ((const float2 *) abl_NB.cols[0])[abl_pslot2];
                }
                Prey* prey = &abl_nx2;
                {
                    const auto separation = abl::make_lazy_dist(abl_q2, abl_NB, abl_slot2, [&]() -> abl_float { return length_float2(float2_sub(in->pos, prey->pos)); });
                    group_center = float2_add(group_center, prey->pos);
                    group_centre_count += 1;
                    if (((separation < abl_G.SAME_SPECIES_AVOIDANCE_RADIUS) && float2_not_equals(prey->pos, in->pos))) abl_dm2_0 |= 1ull << abl_k;
                }
            }
            for (unsigned long long abl_m = abl_dm2_0; abl_m; abl_m &= abl_m - 1ull) {
                const int abl_slot2 = abl_c2.slot(__ffsll((long long) abl_m) - 1);
                Prey abl_nx2;
                abl_nx2.pos = ((const float2 *) abl_NB.cols[0])[abl_slot2];
                Prey* prey = &abl_nx2;
                double separation = length_float2(float2_sub(in->pos, prey->pos));
                {
                    if ((separation > 0.0)) {
                        avoid_velocity = float2_add(avoid_velocity, float2_mul_scalar(float2_sub(in->pos, prey->pos), (abl_G.SAME_SPECIES_AVOIDANCE_RADIUS / separation)));
                    }
                }
            }
        }
    }
    if ((group_centre_count > 0)) {
        group_center = float2_div_scalar(group_center, group_centre_count);
        group_velocity = float2_sub(group_center, in->pos);
    }
    out->steer = float2_add(float2_add(in->steer, group_velocity), avoid_velocity);
}

#ifndef ABL_PERSIST
struct abl_kargs_prey_flock {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Prey in, out;
    abl_near_view NB;
    uint8_t *removed;
    uint8_t *child_flag;
    void *child_cols[ABL_MAX_MEMBERS];
    uint64_t seed;
    long timestep;
    int step_index;
    uint32_t skip_store;
    unsigned long long *serial_rng;
};
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_prey_flock(const __grid_constant__ abl_kargs_prey_flock A) {
    int abl_j;
    {
        const abl_globals &abl_G = A.G;
        const long abl_t1 = (long) blockIdx.x * blockDim.x + threadIdx.x;
        const bool abl_has = abl_t1 < A.n;
        const long abl_i1 = abl_has ? (A.visit ? (long) A.visit[abl_t1] : abl_t1) : 0;
        const float2 abl_p1 = abl_has ? A.in.pos[abl_i1] : float2{};
        const abl::near_query<2> abl_q0(A.NB, (double) abl_p1.x, (double) abl_p1.y, 0.0, abl_has ? abl_i1 : -1);
        auto abl_x0 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) A.NB.cols[0])[abl_s];
            return !(dist_float2(abl_p, abl_p1) > abl_G.PREY_GROUP_COHESION_RADIUS);
        };
        abl_j = abl::presort_block<2>(A.NB, abl_has, abl_q0, abl_x0);
    }
    const long abl_t = (long) blockIdx.x * blockDim.x + abl_j;
    if (abl_t >= A.n) return;
    const long abl_i = A.visit ? (long) A.visit[abl_t] : abl_t;
    abl::step_ctx abl_K;
    abl_K.R.init(A.seed, (uint32_t) abl_i, (uint32_t) A.step_index, (uint64_t) A.timestep);
    abl_K.R.xs = A.serial_rng;
    abl_K.self = abl_i;
    abl_K.removed = 0;
    abl_K.added = 0;
    abl_K.child_cols = A.child_cols;
    abl_K.near_col = abl_j;
    Prey abl_in, abl_out;
    abl_in.pos = A.in.pos[abl_i];
    abl_in.dir = A.in.dir[abl_i];
    abl_in.steer = A.in.steer[abl_i];
    abl_in.life = A.in.life[abl_i];
    abl_out = abl_in;
    prey_flock(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.pos[abl_i] = abl_out.pos;
    A.out.dir[abl_i] = abl_out.dir;
    A.out.steer[abl_i] = abl_out.steer;
    A.out.life[abl_i] = abl_out.life;
}
static int abl_launch_prey_flock(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_prey_flock A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.pos = (float2 *) L->in_cols[0];
    A.out.pos = (float2 *) L->out_cols[0];
    A.in.dir = (float2 *) L->in_cols[1];
    A.out.dir = (float2 *) L->out_cols[1];
    A.in.steer = (float2 *) L->in_cols[2];
    A.out.steer = (float2 *) L->out_cols[2];
    A.in.life = (int *) L->in_cols[3];
    A.out.life = (int *) L->out_cols[3];
    A.NB = L->near;
    A.removed = L->removed;
    A.child_flag = L->child_flag;
    for (int k = 0; k < ABL_MAX_MEMBERS; k++) A.child_cols[k] = L->child_cols[k];
    A.seed = L->seed;
    A.timestep = L->timestep;
    A.step_index = L->step_index;
    A.skip_store = L->skip_store;
    A.serial_rng = L->serial_rng;
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (A.n + abl_block - 1) / abl_block;
    abl_kernel_prey_flock<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
__device__ __forceinline__ void abl_ens_body_prey_flock(const abl_ens_launch &A, long abl_vb, long abl_ts) {
    int abl_j;
    {
        const long abl_t1 = abl_vb * blockDim.x + threadIdx.x;
        const bool abl_has = abl_t1 < A.n;
        const long abl_i1 = abl_has ? (A.visit_order ? (long) A.visit_order[abl_t1] : abl_t1) : 0;
        const int abl_r1 = abl_has ? A.replica[abl_i1] : 0;
        const abl_globals &abl_G = ((const abl_globals *) A.globals)[abl_r1];
        const abl_near_view &abl_V1 = A.views[abl_r1];
        const float2 abl_p1 = abl_has ? ((const float2 *) A.in_cols[0])[abl_i1] : float2{};
        const abl::near_query<2> abl_q0(abl_V1, (double) abl_p1.x, (double) abl_p1.y, 0.0, abl_has ? abl_i1 : -1);
        auto abl_x0 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) abl_V1.cols[0])[abl_s];
            return !(dist_float2(abl_p, abl_p1) > abl_G.PREY_GROUP_COHESION_RADIUS);
        };
        abl_j = abl::presort_block<2>(abl_V1, abl_has, abl_q0, abl_x0);
    }
    const long abl_t = abl_vb * blockDim.x + abl_j;
    if (abl_t >= A.n) return;
    const long abl_i = A.visit_order ? (long) A.visit_order[abl_t] : abl_t;
    const int abl_r = A.replica[abl_i];
    const abl_globals &abl_Gr = ((const abl_globals *) A.globals)[abl_r];
    abl::step_ctx abl_K;
    abl_K.R.init(A.seeds[abl_r], (uint32_t) (abl_i - A.agent_base[abl_r]), (uint32_t) A.step_index, (uint64_t) abl_ts);
    abl_K.self = abl_i;
    abl_K.removed = 0;
    abl_K.added = 0;
    abl_K.child_cols = nullptr;
    abl_K.near_col = abl_j;
    Prey abl_in, abl_out;
    abl_in.pos = ((const float2 *) A.in_cols[0])[abl_i];
    abl_in.dir = ((const float2 *) A.in_cols[1])[abl_i];
    abl_in.steer = ((const float2 *) A.in_cols[2])[abl_i];
    abl_in.life = ((const int *) A.in_cols[3])[abl_i];
    abl_out.pos = abl_in.pos;
    abl_out.dir = abl_in.dir;
    abl_out.steer = abl_in.steer;
    abl_out.life = abl_in.life;
    prey_flock(abl_Gr, A.views[abl_r], abl_K, &abl_in, &abl_out);
    ((float2 *) A.out_cols[0])[abl_i] = abl_out.pos;
    ((float2 *) A.out_cols[1])[abl_i] = abl_out.dir;
    ((float2 *) A.out_cols[2])[abl_i] = abl_out.steer;
    ((int *) A.out_cols[3])[abl_i] = abl_out.life;
}
#ifndef ABL_PERSIST
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ens_prey_flock(const __grid_constant__ abl_ens_launch A) {
    abl_ens_body_prey_flock(A, blockIdx.x, A.timestep);
}
static int abl_launch_ens_prey_flock(const abl_ens_launch *L, cudaStream_t abl_stream) {
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (L->n + abl_block - 1) / abl_block;
    abl_kernel_ens_prey_flock<<<abl_grid, abl_block, L->smem, abl_stream>>>(*L);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
#ifndef ABL_PERSIST
static double abl_radius_prey_flock(const void *abl_gp) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    return (double) (abl_G.PREY_GROUP_COHESION_RADIUS);
}
#endif

__device__ static void prey_move(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Prey* in, Prey* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    float2 agent_position = in->pos;
    float2 agent_velocity = in->dir;
    float2 agent_steer = in->steer;
    agent_velocity = float2_add(agent_velocity, agent_steer);
    double current_speed = length_float2(agent_velocity);
    if ((current_speed > 1.0)) agent_velocity = normalize_float2(agent_velocity);
    agent_position = float2_add(agent_position, float2_mul_scalar(float2_mul_scalar(agent_velocity, abl_G.DELTA_TIME), abl_G.SPACE_MULT));
    agent_position = boundPosition(abl_G, abl_R, agent_position);
    out->pos = agent_position;
    out->dir = agent_velocity;
    out->life = (in->life - 1);
}

#ifndef ABL_PERSIST
struct abl_kargs_prey_move {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Prey in, out;
    abl_near_view NB;
    uint8_t *removed;
    uint8_t *child_flag;
    void *child_cols[ABL_MAX_MEMBERS];
    uint64_t seed;
    long timestep;
    int step_index;
    uint32_t skip_store;
    unsigned long long *serial_rng;
};
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_prey_move(const __grid_constant__ abl_kargs_prey_move A) {
    const long abl_t = (long) blockIdx.x * blockDim.x + threadIdx.x;
    if (abl_t >= A.n) return;
    const long abl_i = A.visit ? (long) A.visit[abl_t] : abl_t;
    abl::step_ctx abl_K;
    abl_K.R.init(A.seed, (uint32_t) abl_i, (uint32_t) A.step_index, (uint64_t) A.timestep);
    abl_K.R.xs = A.serial_rng;
    abl_K.self = abl_i;
    abl_K.removed = 0;
    abl_K.added = 0;
    abl_K.child_cols = A.child_cols;
    abl_K.near_col = -1;
    Prey abl_in, abl_out;
    abl_in.pos = A.in.pos[abl_i];
    abl_in.dir = A.in.dir[abl_i];
    abl_in.steer = A.in.steer[abl_i];
    abl_in.life = A.in.life[abl_i];
    abl_out = abl_in;
    prey_move(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.pos[abl_i] = abl_out.pos;
    A.out.dir[abl_i] = abl_out.dir;
    A.out.steer[abl_i] = abl_out.steer;
    A.out.life[abl_i] = abl_out.life;
}
static int abl_launch_prey_move(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_prey_move A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.pos = (float2 *) L->in_cols[0];
    A.out.pos = (float2 *) L->out_cols[0];
    A.in.dir = (float2 *) L->in_cols[1];
    A.out.dir = (float2 *) L->out_cols[1];
    A.in.steer = (float2 *) L->in_cols[2];
    A.out.steer = (float2 *) L->out_cols[2];
    A.in.life = (int *) L->in_cols[3];
    A.out.life = (int *) L->out_cols[3];
    A.NB = L->near;
    A.removed = L->removed;
    A.child_flag = L->child_flag;
    for (int k = 0; k < ABL_MAX_MEMBERS; k++) A.child_cols[k] = L->child_cols[k];
    A.seed = L->seed;
    A.timestep = L->timestep;
    A.step_index = L->step_index;
    A.skip_store = L->skip_store;
    A.serial_rng = L->serial_rng;
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (A.n + abl_block - 1) / abl_block;
    abl_kernel_prey_move<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
__device__ __forceinline__ void abl_ens_body_prey_move(const abl_ens_launch &A, long abl_vb, long abl_ts) {
    const long abl_t = abl_vb * blockDim.x + threadIdx.x;
    if (abl_t >= A.n) return;
    const long abl_i = A.visit_order ? (long) A.visit_order[abl_t] : abl_t;
    const int abl_r = A.replica[abl_i];
    const abl_globals &abl_Gr = ((const abl_globals *) A.globals)[abl_r];
    abl::step_ctx abl_K;
    abl_K.R.init(A.seeds[abl_r], (uint32_t) (abl_i - A.agent_base[abl_r]), (uint32_t) A.step_index, (uint64_t) abl_ts);
    abl_K.self = abl_i;
    abl_K.removed = 0;
    abl_K.added = 0;
    abl_K.child_cols = nullptr;
    abl_K.near_col = -1;
    Prey abl_in, abl_out;
    abl_in.pos = ((const float2 *) A.in_cols[0])[abl_i];
    abl_in.dir = ((const float2 *) A.in_cols[1])[abl_i];
    abl_in.steer = ((const float2 *) A.in_cols[2])[abl_i];
    abl_in.life = ((const int *) A.in_cols[3])[abl_i];
    abl_out.pos = abl_in.pos;
    abl_out.dir = abl_in.dir;
    abl_out.steer = abl_in.steer;
    abl_out.life = abl_in.life;
    prey_move(abl_Gr, A.views[abl_r], abl_K, &abl_in, &abl_out);
    ((float2 *) A.out_cols[0])[abl_i] = abl_out.pos;
    ((float2 *) A.out_cols[1])[abl_i] = abl_out.dir;
    ((float2 *) A.out_cols[2])[abl_i] = abl_out.steer;
    ((int *) A.out_cols[3])[abl_i] = abl_out.life;
}
#ifndef ABL_PERSIST
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ens_prey_move(const __grid_constant__ abl_ens_launch A) {
    abl_ens_body_prey_move(A, blockIdx.x, A.timestep);
}
static int abl_launch_ens_prey_move(const abl_ens_launch *L, cudaStream_t abl_stream) {
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (L->n + abl_block - 1) / abl_block;
    abl_kernel_ens_prey_move<<<abl_grid, abl_block, L->smem, abl_stream>>>(*L);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif

__device__ static void prey_eaten(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Prey* in, Prey* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    bool eaten = false;
    double closest_pred = abl_G.PRED_KILL_DISTANCE;
    {
        const abl::near_query<2> abl_q3(abl_NB, (double) in->pos.x, (double) in->pos.y, 0.0, abl_K.self);
        abl::near_list_cursor<2> abl_c3(abl_NB, abl_q3, abl_K);
        auto abl_exact3 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) abl_NB.cols[0])[abl_s];
            return !(dist_float2(abl_p, in->pos) > abl_G.PRED_KILL_DISTANCE);
        };
        while (abl_c3.fill(abl_q3, abl_exact3)) {
            int abl_pslot3 = abl_c3.slot(0);
            Predator abl_pnx3;
            abl_pnx3.pos = ((const float2 *) abl_NB.cols[0])[abl_pslot3];
            for (int abl_k = 0; abl_k < abl_c3.cnt; ++abl_k) {
                const int abl_slot3 = abl_pslot3;
                Predator abl_nx3 = abl_pnx3;
                if (abl_k + 1 < abl_c3.cnt) {
                    abl_pslot3 = abl_c3.slot(abl_k + 1);
                    abl_pnx3.pos = ((const float2 *) abl_NB.cols[0])[abl_pslot3];
                }
                Predator* pred = &abl_nx3;
                {
                    double distance = length_float2(float2_sub(pred->pos, in->pos));
                    if ((distance < closest_pred)) {
                        closest_pred = distance;
                        eaten = true;
                    }
                }
            }
        }
    }
    if (eaten) abl_K.remove();
}

#ifndef ABL_PERSIST
struct abl_kargs_prey_eaten {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Prey in, out;
    abl_near_view NB;
    uint8_t *removed;
    uint8_t *child_flag;
    void *child_cols[ABL_MAX_MEMBERS];
    uint64_t seed;
    long timestep;
    int step_index;
    uint32_t skip_store;
    unsigned long long *serial_rng;
};
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_prey_eaten(const __grid_constant__ abl_kargs_prey_eaten A) {
    int abl_j;
    {
        const abl_globals &abl_G = A.G;
        const long abl_t1 = (long) blockIdx.x * blockDim.x + threadIdx.x;
        const bool abl_has = abl_t1 < A.n;
        const long abl_i1 = abl_has ? (A.visit ? (long) A.visit[abl_t1] : abl_t1) : 0;
        const float2 abl_p1 = abl_has ? A.in.pos[abl_i1] : float2{};
        const abl::near_query<2> abl_q0(A.NB, (double) abl_p1.x, (double) abl_p1.y, 0.0, abl_has ? abl_i1 : -1);
        auto abl_x0 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) A.NB.cols[0])[abl_s];
            return !(dist_float2(abl_p, abl_p1) > abl_G.PRED_KILL_DISTANCE);
        };
        abl_j = abl::presort_block<2>(A.NB, abl_has, abl_q0, abl_x0);
    }
    const long abl_t = (long) blockIdx.x * blockDim.x + abl_j;
    if (abl_t >= A.n) return;
    const long abl_i = A.visit ? (long) A.visit[abl_t] : abl_t;
    abl::step_ctx abl_K;
    abl_K.R.init(A.seed, (uint32_t) abl_i, (uint32_t) A.step_index, (uint64_t) A.timestep);
    abl_K.R.xs = A.serial_rng;
    abl_K.self = abl_i;
    abl_K.removed = 0;
    abl_K.added = 0;
    abl_K.child_cols = A.child_cols;
    abl_K.near_col = abl_j;
    Prey abl_in, abl_out;
    abl_in.pos = A.in.pos[abl_i];
    abl_in.dir = A.in.dir[abl_i];
    abl_in.steer = A.in.steer[abl_i];
    abl_in.life = A.in.life[abl_i];
    abl_out = abl_in;
    prey_eaten(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.pos[abl_i] = abl_out.pos;
    A.out.dir[abl_i] = abl_out.dir;
    A.out.steer[abl_i] = abl_out.steer;
    A.out.life[abl_i] = abl_out.life;
    A.removed[abl_i] = (uint8_t) abl_K.removed;
}
static int abl_launch_prey_eaten(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_prey_eaten A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.pos = (float2 *) L->in_cols[0];
    A.out.pos = (float2 *) L->out_cols[0];
    A.in.dir = (float2 *) L->in_cols[1];
    A.out.dir = (float2 *) L->out_cols[1];
    A.in.steer = (float2 *) L->in_cols[2];
    A.out.steer = (float2 *) L->out_cols[2];
    A.in.life = (int *) L->in_cols[3];
    A.out.life = (int *) L->out_cols[3];
    A.NB = L->near;
    A.removed = L->removed;
    A.child_flag = L->child_flag;
    for (int k = 0; k < ABL_MAX_MEMBERS; k++) A.child_cols[k] = L->child_cols[k];
    A.seed = L->seed;
    A.timestep = L->timestep;
    A.step_index = L->step_index;
    A.skip_store = L->skip_store;
    A.serial_rng = L->serial_rng;
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (A.n + abl_block - 1) / abl_block;
    abl_kernel_prey_eaten<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
#ifndef ABL_PERSIST
static double abl_radius_prey_eaten(const void *abl_gp) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    return (double) (abl_G.PRED_KILL_DISTANCE);
}
#endif

__device__ static void prey_eat_or_starve(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Prey* in, Prey* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    int life = in->life;
    {
        const abl::near_query<2> abl_q4(abl_NB, (double) in->pos.x, (double) in->pos.y, 0.0, abl_K.self);
        abl::near_cursor<2> abl_c4(abl_NB, abl_q4);
        auto abl_exact4 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) abl_NB.cols[0])[abl_s];
            return !(dist_float2(abl_p, in->pos) > abl_G.GRASS_EAT_DISTANCE);
        };
        while (abl_c4.fill(abl_q4, abl_exact4)) {
            int abl_pslot4 = abl_c4.slot(0);
            Grass abl_pnx4;
            abl_pnx4.avail = ((const bool *) abl_NB.cols[2])[abl_pslot4];
            for (int abl_k = 0; abl_k < abl_c4.cnt; ++abl_k) {
                const int abl_slot4 = abl_pslot4;
                Grass abl_nx4 = abl_pnx4;
                if (abl_k + 1 < abl_c4.cnt) {
                    abl_pslot4 = abl_c4.slot(abl_k + 1);
                    abl_pnx4.avail = ((const bool *) abl_NB.cols[2])[abl_pslot4];
                }
                Grass* grass = &abl_nx4;
                {
                    if (grass->avail) life += abl_G.GAIN_FROM_FOOD_PREY;
                }
            }
        }
    }
    out->life = life;
    if ((life < 1)) abl_K.remove();
}

#ifndef ABL_PERSIST
struct abl_kargs_prey_eat_or_starve {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Prey in, out;
    abl_near_view NB;
    uint8_t *removed;
    uint8_t *child_flag;
    void *child_cols[ABL_MAX_MEMBERS];
    uint64_t seed;
    long timestep;
    int step_index;
    uint32_t skip_store;
    unsigned long long *serial_rng;
};
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_prey_eat_or_starve(const __grid_constant__ abl_kargs_prey_eat_or_starve A) {
    const long abl_t = (long) blockIdx.x * blockDim.x + threadIdx.x;
    if (abl_t >= A.n) return;
    const long abl_i = A.visit ? (long) A.visit[abl_t] : abl_t;
    abl::step_ctx abl_K;
    abl_K.R.init(A.seed, (uint32_t) abl_i, (uint32_t) A.step_index, (uint64_t) A.timestep);
    abl_K.R.xs = A.serial_rng;
    abl_K.self = abl_i;
    abl_K.removed = 0;
    abl_K.added = 0;
    abl_K.child_cols = A.child_cols;
    abl_K.near_col = -1;
    Prey abl_in, abl_out;
    abl_in.pos = A.in.pos[abl_i];
    abl_in.dir = A.in.dir[abl_i];
    abl_in.steer = A.in.steer[abl_i];
    abl_in.life = A.in.life[abl_i];
    abl_out = abl_in;
    prey_eat_or_starve(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.pos[abl_i] = abl_out.pos;
    A.out.dir[abl_i] = abl_out.dir;
    A.out.steer[abl_i] = abl_out.steer;
    A.out.life[abl_i] = abl_out.life;
    A.removed[abl_i] = (uint8_t) abl_K.removed;
}
static int abl_launch_prey_eat_or_starve(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_prey_eat_or_starve A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.pos = (float2 *) L->in_cols[0];
    A.out.pos = (float2 *) L->out_cols[0];
    A.in.dir = (float2 *) L->in_cols[1];
    A.out.dir = (float2 *) L->out_cols[1];
    A.in.steer = (float2 *) L->in_cols[2];
    A.out.steer = (float2 *) L->out_cols[2];
    A.in.life = (int *) L->in_cols[3];
    A.out.life = (int *) L->out_cols[3];
    A.NB = L->near;
    A.removed = L->removed;
    A.child_flag = L->child_flag;
    for (int k = 0; k < ABL_MAX_MEMBERS; k++) A.child_cols[k] = L->child_cols[k];
    A.seed = L->seed;
    A.timestep = L->timestep;
    A.step_index = L->step_index;
    A.skip_store = L->skip_store;
    A.serial_rng = L->serial_rng;
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (A.n + abl_block - 1) / abl_block;
    abl_kernel_prey_eat_or_starve<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
#ifndef ABL_PERSIST
static double abl_radius_prey_eat_or_starve(const void *abl_gp) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    return (double) (abl_G.GRASS_EAT_DISTANCE);
}
#endif

__device__ static void prey_reproduction(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Prey* in, Prey* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    if ((random_3(abl_G, abl_R, 1.0) < abl_G.REPRODUCE_PREY_PROB)) {
        abl_add_Prey(abl_K, ([&]() { Prey abl_a; abl_a.pos = in->pos; abl_a.dir = float2_mul_scalar(in->dir, -1.0); abl_a.steer = float2_mul_scalar(in->steer, -1.0); abl_a.life = (in->life / 2); return abl_a; }()));
        out->life = (in->life / 2);
    }
}

#ifndef ABL_PERSIST
struct abl_kargs_prey_reproduction {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Prey in, out;
    abl_near_view NB;
    uint8_t *removed;
    uint8_t *child_flag;
    void *child_cols[ABL_MAX_MEMBERS];
    uint64_t seed;
    long timestep;
    int step_index;
    uint32_t skip_store;
    unsigned long long *serial_rng;
};
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_prey_reproduction(const __grid_constant__ abl_kargs_prey_reproduction A) {
    const long abl_t = (long) blockIdx.x * blockDim.x + threadIdx.x;
    if (abl_t >= A.n) return;
    const long abl_i = A.visit ? (long) A.visit[abl_t] : abl_t;
    abl::step_ctx abl_K;
    abl_K.R.init(A.seed, (uint32_t) abl_i, (uint32_t) A.step_index, (uint64_t) A.timestep);
    abl_K.R.xs = A.serial_rng;
    abl_K.self = abl_i;
    abl_K.removed = 0;
    abl_K.added = 0;
    abl_K.child_cols = A.child_cols;
    abl_K.near_col = -1;
    Prey abl_in, abl_out;
    abl_in.pos = A.in.pos[abl_i];
    abl_in.dir = A.in.dir[abl_i];
    abl_in.steer = A.in.steer[abl_i];
    abl_in.life = A.in.life[abl_i];
    abl_out = abl_in;
    prey_reproduction(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.pos[abl_i] = abl_out.pos;
    A.out.dir[abl_i] = abl_out.dir;
    A.out.steer[abl_i] = abl_out.steer;
    A.out.life[abl_i] = abl_out.life;
    A.child_flag[abl_i] = (uint8_t) abl_K.added;
}
static int abl_launch_prey_reproduction(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_prey_reproduction A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.pos = (float2 *) L->in_cols[0];
    A.out.pos = (float2 *) L->out_cols[0];
    A.in.dir = (float2 *) L->in_cols[1];
    A.out.dir = (float2 *) L->out_cols[1];
    A.in.steer = (float2 *) L->in_cols[2];
    A.out.steer = (float2 *) L->out_cols[2];
    A.in.life = (int *) L->in_cols[3];
    A.out.life = (int *) L->out_cols[3];
    A.NB = L->near;
    A.removed = L->removed;
    A.child_flag = L->child_flag;
    for (int k = 0; k < ABL_MAX_MEMBERS; k++) A.child_cols[k] = L->child_cols[k];
    A.seed = L->seed;
    A.timestep = L->timestep;
    A.step_index = L->step_index;
    A.skip_store = L->skip_store;
    A.serial_rng = L->serial_rng;
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (A.n + abl_block - 1) / abl_block;
    abl_kernel_prey_reproduction<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif

__device__ static void pred_follow_prey(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Predator* in, Predator* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    float2 agent_position = in->pos;
    float2 agent_steer = float2_create(0, 0);
    float2 closest_prey_position = float2_create(0, 0);
    double closest_prey_distance = abl_G.PRED_PREY_INTERACTION_RADIUS;
    bool can_see_prey = false;
    {
        const abl::near_query<2> abl_q5(abl_NB, (double) in->pos.x, (double) in->pos.y, 0.0, abl_K.self);
        abl::near_list_cursor<2> abl_c5(abl_NB, abl_q5, abl_K);
        auto abl_exact5 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) abl_NB.cols[0])[abl_s];
            return !(dist_float2(abl_p, in->pos) > abl_G.PRED_PREY_INTERACTION_RADIUS);
        };
        while (abl_c5.fill(abl_q5, abl_exact5)) {
            int abl_pslot5 = abl_c5.slot(0);
            Prey abl_pnx5;
            abl_pnx5.pos = ((const float2 *) abl_NB.cols[0])[abl_pslot5];
            for (int abl_k = 0; abl_k < abl_c5.cnt; ++abl_k) {
                const int abl_slot5 = abl_pslot5;
                Prey abl_nx5 = abl_pnx5;
                if (abl_k + 1 < abl_c5.cnt) {
                    abl_pslot5 = abl_c5.slot(abl_k + 1);
                    abl_pnx5.pos = ((const float2 *) abl_NB.cols[0])[abl_pslot5];
                }
                Prey* prey = &abl_nx5;
                {
                    double separation = length_float2(float2_sub(in->pos, prey->pos));
                    if ((separation < closest_prey_distance)) {
                        closest_prey_position = prey->pos;
                        closest_prey_distance = separation;
                        can_see_prey = true;
                    }
                }
            }
        }
    }
    if (can_see_prey) {
        agent_steer = float2_sub(closest_prey_position, agent_position);
    }
    out->steer = agent_steer;
}

#ifndef ABL_PERSIST
struct abl_kargs_pred_follow_prey {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Predator in, out;
    abl_near_view NB;
    uint8_t *removed;
    uint8_t *child_flag;
    void *child_cols[ABL_MAX_MEMBERS];
    uint64_t seed;
    long timestep;
    int step_index;
    uint32_t skip_store;
    unsigned long long *serial_rng;
};
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_pred_follow_prey(const __grid_constant__ abl_kargs_pred_follow_prey A) {
    int abl_j;
    {
        const abl_globals &abl_G = A.G;
        const long abl_t1 = (long) blockIdx.x * blockDim.x + threadIdx.x;
        const bool abl_has = abl_t1 < A.n;
        const long abl_i1 = abl_has ? (A.visit ? (long) A.visit[abl_t1] : abl_t1) : 0;
        const float2 abl_p1 = abl_has ? A.in.pos[abl_i1] : float2{};
        const abl::near_query<2> abl_q0(A.NB, (double) abl_p1.x, (double) abl_p1.y, 0.0, abl_has ? abl_i1 : -1);
        auto abl_x0 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) A.NB.cols[0])[abl_s];
            return !(dist_float2(abl_p, abl_p1) > abl_G.PRED_PREY_INTERACTION_RADIUS);
        };
        abl_j = abl::presort_block<2>(A.NB, abl_has, abl_q0, abl_x0);
    }
    const long abl_t = (long) blockIdx.x * blockDim.x + abl_j;
    if (abl_t >= A.n) return;
    const long abl_i = A.visit ? (long) A.visit[abl_t] : abl_t;
    abl::step_ctx abl_K;
    abl_K.R.init(A.seed, (uint32_t) abl_i, (uint32_t) A.step_index, (uint64_t) A.timestep);
    abl_K.R.xs = A.serial_rng;
    abl_K.self = abl_i;
    abl_K.removed = 0;
    abl_K.added = 0;
    abl_K.child_cols = A.child_cols;
    abl_K.near_col = abl_j;
    Predator abl_in, abl_out;
    abl_in.pos = A.in.pos[abl_i];
    abl_in.dir = A.in.dir[abl_i];
    abl_in.steer = A.in.steer[abl_i];
    abl_in.life = A.in.life[abl_i];
    abl_out = abl_in;
    pred_follow_prey(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.pos[abl_i] = abl_out.pos;
    A.out.dir[abl_i] = abl_out.dir;
    A.out.steer[abl_i] = abl_out.steer;
    A.out.life[abl_i] = abl_out.life;
}
static int abl_launch_pred_follow_prey(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_pred_follow_prey A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.pos = (float2 *) L->in_cols[0];
    A.out.pos = (float2 *) L->out_cols[0];
    A.in.dir = (float2 *) L->in_cols[1];
    A.out.dir = (float2 *) L->out_cols[1];
    A.in.steer = (float2 *) L->in_cols[2];
    A.out.steer = (float2 *) L->out_cols[2];
    A.in.life = (int *) L->in_cols[3];
    A.out.life = (int *) L->out_cols[3];
    A.NB = L->near;
    A.removed = L->removed;
    A.child_flag = L->child_flag;
    for (int k = 0; k < ABL_MAX_MEMBERS; k++) A.child_cols[k] = L->child_cols[k];
    A.seed = L->seed;
    A.timestep = L->timestep;
    A.step_index = L->step_index;
    A.skip_store = L->skip_store;
    A.serial_rng = L->serial_rng;
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (A.n + abl_block - 1) / abl_block;
    abl_kernel_pred_follow_prey<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
__device__ __forceinline__ void abl_ens_body_pred_follow_prey(const abl_ens_launch &A, long abl_vb, long abl_ts) {
    int abl_j;
    {
        const long abl_t1 = abl_vb * blockDim.x + threadIdx.x;
        const bool abl_has = abl_t1 < A.n;
        const long abl_i1 = abl_has ? (A.visit_order ? (long) A.visit_order[abl_t1] : abl_t1) : 0;
        const int abl_r1 = abl_has ? A.replica[abl_i1] : 0;
        const abl_globals &abl_G = ((const abl_globals *) A.globals)[abl_r1];
        const abl_near_view &abl_V1 = A.views[abl_r1];
        const float2 abl_p1 = abl_has ? ((const float2 *) A.in_cols[0])[abl_i1] : float2{};
        const abl::near_query<2> abl_q0(abl_V1, (double) abl_p1.x, (double) abl_p1.y, 0.0, abl_has ? abl_i1 : -1);
        auto abl_x0 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) abl_V1.cols[0])[abl_s];
            return !(dist_float2(abl_p, abl_p1) > abl_G.PRED_PREY_INTERACTION_RADIUS);
        };
        abl_j = abl::presort_block<2>(abl_V1, abl_has, abl_q0, abl_x0);
    }
    const long abl_t = abl_vb * blockDim.x + abl_j;
    if (abl_t >= A.n) return;
    const long abl_i = A.visit_order ? (long) A.visit_order[abl_t] : abl_t;
    const int abl_r = A.replica[abl_i];
    const abl_globals &abl_Gr = ((const abl_globals *) A.globals)[abl_r];
    abl::step_ctx abl_K;
    abl_K.R.init(A.seeds[abl_r], (uint32_t) (abl_i - A.agent_base[abl_r]), (uint32_t) A.step_index, (uint64_t) abl_ts);
    abl_K.self = abl_i;
    abl_K.removed = 0;
    abl_K.added = 0;
    abl_K.child_cols = nullptr;
    abl_K.near_col = abl_j;
    Predator abl_in, abl_out;
    abl_in.pos = ((const float2 *) A.in_cols[0])[abl_i];
    abl_in.dir = ((const float2 *) A.in_cols[1])[abl_i];
    abl_in.steer = ((const float2 *) A.in_cols[2])[abl_i];
    abl_in.life = ((const int *) A.in_cols[3])[abl_i];
    abl_out.pos = abl_in.pos;
    abl_out.dir = abl_in.dir;
    abl_out.steer = abl_in.steer;
    abl_out.life = abl_in.life;
    pred_follow_prey(abl_Gr, A.views[abl_r], abl_K, &abl_in, &abl_out);
    ((float2 *) A.out_cols[0])[abl_i] = abl_out.pos;
    ((float2 *) A.out_cols[1])[abl_i] = abl_out.dir;
    ((float2 *) A.out_cols[2])[abl_i] = abl_out.steer;
    ((int *) A.out_cols[3])[abl_i] = abl_out.life;
}
#ifndef ABL_PERSIST
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ens_pred_follow_prey(const __grid_constant__ abl_ens_launch A) {
    abl_ens_body_pred_follow_prey(A, blockIdx.x, A.timestep);
}
static int abl_launch_ens_pred_follow_prey(const abl_ens_launch *L, cudaStream_t abl_stream) {
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (L->n + abl_block - 1) / abl_block;
    abl_kernel_ens_pred_follow_prey<<<abl_grid, abl_block, L->smem, abl_stream>>>(*L);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
#ifndef ABL_PERSIST
static double abl_radius_pred_follow_prey(const void *abl_gp) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    return (double) (abl_G.PRED_PREY_INTERACTION_RADIUS);
}
#endif

__device__ static void pred_avoid(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Predator* in, Predator* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    float2 avoid_velocity = float2_create(0, 0);
    {
        const abl::near_query<2> abl_q6(abl_NB, (double) in->pos.x, (double) in->pos.y, 0.0, abl_K.self);
        abl::near_list_cursor<2> abl_c6(abl_NB, abl_q6, abl_K);
        auto abl_exact6 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) abl_NB.cols[0])[abl_s];
            return !(dist_float2(abl_p, in->pos) > abl_G.SAME_SPECIES_AVOIDANCE_RADIUS);
        };
        while (abl_c6.fill(abl_q6, abl_exact6)) {
            int abl_pslot6 = abl_c6.slot(0);
            Predator abl_pnx6;
            abl_pnx6.pos = ((const float2 *) abl_NB.cols[0])[abl_pslot6];
            unsigned long long abl_dm6_0 = 0ull;
            for (int abl_k = 0; abl_k < abl_c6.cnt; ++abl_k) {
                const int abl_slot6 = abl_pslot6;
                Predator abl_nx6 = abl_pnx6;
                if (abl_k + 1 < abl_c6.cnt) {
                    abl_pslot6 = abl_c6.slot(abl_k + 1);
                    abl_pnx6.pos = ((const float2 *) abl_NB.cols[0])[abl_pslot6];
                }
                Predator* pred = &abl_nx6;
                {
                    const auto separation = abl::make_lazy_dist(abl_q6, abl_NB, abl_slot6, [&]() -> abl_float { return length_float2(float2_sub(in->pos, pred->pos)); });
                    if (((separation < abl_G.SAME_SPECIES_AVOIDANCE_RADIUS) && float2_not_equals(pred->pos, in->pos))) abl_dm6_0 |= 1ull << abl_k;
                }
            }
            for (unsigned long long abl_m = abl_dm6_0; abl_m; abl_m &= abl_m - 1ull) {
                const int abl_slot6 = abl_c6.slot(__ffsll((long long) abl_m) - 1);
                Predator abl_nx6;
                abl_nx6.pos = ((const float2 *) abl_NB.cols[0])[abl_slot6];
                Predator* pred = &abl_nx6;
                double separation = length_float2(float2_sub(in->pos, pred->pos));
                {
                    if ((separation > 0.0)) avoid_velocity = float2_add(avoid_velocity, float2_mul_scalar(float2_sub(in->pos, pred->pos), (abl_G.SAME_SPECIES_AVOIDANCE_RADIUS / separation)));
                }
            }
        }
    }
    out->steer = float2_add(in->steer, avoid_velocity);
}

#ifndef ABL_PERSIST
struct abl_kargs_pred_avoid {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Predator in, out;
    abl_near_view NB;
    uint8_t *removed;
    uint8_t *child_flag;
    void *child_cols[ABL_MAX_MEMBERS];
    uint64_t seed;
    long timestep;
    int step_index;
    uint32_t skip_store;
    unsigned long long *serial_rng;
};
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_pred_avoid(const __grid_constant__ abl_kargs_pred_avoid A) {
    int abl_j;
    {
        const abl_globals &abl_G = A.G;
        const long abl_t1 = (long) blockIdx.x * blockDim.x + threadIdx.x;
        const bool abl_has = abl_t1 < A.n;
        const long abl_i1 = abl_has ? (A.visit ? (long) A.visit[abl_t1] : abl_t1) : 0;
        const float2 abl_p1 = abl_has ? A.in.pos[abl_i1] : float2{};
        const abl::near_query<2> abl_q0(A.NB, (double) abl_p1.x, (double) abl_p1.y, 0.0, abl_has ? abl_i1 : -1);
        auto abl_x0 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) A.NB.cols[0])[abl_s];
            return !(dist_float2(abl_p, abl_p1) > abl_G.SAME_SPECIES_AVOIDANCE_RADIUS);
        };
        abl_j = abl::presort_block<2>(A.NB, abl_has, abl_q0, abl_x0);
    }
    const long abl_t = (long) blockIdx.x * blockDim.x + abl_j;
    if (abl_t >= A.n) return;
    const long abl_i = A.visit ? (long) A.visit[abl_t] : abl_t;
    abl::step_ctx abl_K;
    abl_K.R.init(A.seed, (uint32_t) abl_i, (uint32_t) A.step_index, (uint64_t) A.timestep);
    abl_K.R.xs = A.serial_rng;
    abl_K.self = abl_i;
    abl_K.removed = 0;
    abl_K.added = 0;
    abl_K.child_cols = A.child_cols;
    abl_K.near_col = abl_j;
    Predator abl_in, abl_out;
    abl_in.pos = A.in.pos[abl_i];
    abl_in.dir = A.in.dir[abl_i];
    abl_in.steer = A.in.steer[abl_i];
    abl_in.life = A.in.life[abl_i];
    abl_out = abl_in;
    pred_avoid(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.pos[abl_i] = abl_out.pos;
    A.out.dir[abl_i] = abl_out.dir;
    A.out.steer[abl_i] = abl_out.steer;
    A.out.life[abl_i] = abl_out.life;
}
static int abl_launch_pred_avoid(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_pred_avoid A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.pos = (float2 *) L->in_cols[0];
    A.out.pos = (float2 *) L->out_cols[0];
    A.in.dir = (float2 *) L->in_cols[1];
    A.out.dir = (float2 *) L->out_cols[1];
    A.in.steer = (float2 *) L->in_cols[2];
    A.out.steer = (float2 *) L->out_cols[2];
    A.in.life = (int *) L->in_cols[3];
    A.out.life = (int *) L->out_cols[3];
    A.NB = L->near;
    A.removed = L->removed;
    A.child_flag = L->child_flag;
    for (int k = 0; k < ABL_MAX_MEMBERS; k++) A.child_cols[k] = L->child_cols[k];
    A.seed = L->seed;
    A.timestep = L->timestep;
    A.step_index = L->step_index;
    A.skip_store = L->skip_store;
    A.serial_rng = L->serial_rng;
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (A.n + abl_block - 1) / abl_block;
    abl_kernel_pred_avoid<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
__device__ __forceinline__ void abl_ens_body_pred_avoid(const abl_ens_launch &A, long abl_vb, long abl_ts) {
    int abl_j;
    {
        const long abl_t1 = abl_vb * blockDim.x + threadIdx.x;
        const bool abl_has = abl_t1 < A.n;
        const long abl_i1 = abl_has ? (A.visit_order ? (long) A.visit_order[abl_t1] : abl_t1) : 0;
        const int abl_r1 = abl_has ? A.replica[abl_i1] : 0;
        const abl_globals &abl_G = ((const abl_globals *) A.globals)[abl_r1];
        const abl_near_view &abl_V1 = A.views[abl_r1];
        const float2 abl_p1 = abl_has ? ((const float2 *) A.in_cols[0])[abl_i1] : float2{};
        const abl::near_query<2> abl_q0(abl_V1, (double) abl_p1.x, (double) abl_p1.y, 0.0, abl_has ? abl_i1 : -1);
        auto abl_x0 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) abl_V1.cols[0])[abl_s];
            return !(dist_float2(abl_p, abl_p1) > abl_G.SAME_SPECIES_AVOIDANCE_RADIUS);
        };
        abl_j = abl::presort_block<2>(abl_V1, abl_has, abl_q0, abl_x0);
    }
    const long abl_t = abl_vb * blockDim.x + abl_j;
    if (abl_t >= A.n) return;
    const long abl_i = A.visit_order ? (long) A.visit_order[abl_t] : abl_t;
    const int abl_r = A.replica[abl_i];
    const abl_globals &abl_Gr = ((const abl_globals *) A.globals)[abl_r];
    abl::step_ctx abl_K;
    abl_K.R.init(A.seeds[abl_r], (uint32_t) (abl_i - A.agent_base[abl_r]), (uint32_t) A.step_index, (uint64_t) abl_ts);
    abl_K.self = abl_i;
    abl_K.removed = 0;
    abl_K.added = 0;
    abl_K.child_cols = nullptr;
    abl_K.near_col = abl_j;
    Predator abl_in, abl_out;
    abl_in.pos = ((const float2 *) A.in_cols[0])[abl_i];
    abl_in.dir = ((const float2 *) A.in_cols[1])[abl_i];
    abl_in.steer = ((const float2 *) A.in_cols[2])[abl_i];
    abl_in.life = ((const int *) A.in_cols[3])[abl_i];
    abl_out.pos = abl_in.pos;
    abl_out.dir = abl_in.dir;
    abl_out.steer = abl_in.steer;
    abl_out.life = abl_in.life;
    pred_avoid(abl_Gr, A.views[abl_r], abl_K, &abl_in, &abl_out);
    ((float2 *) A.out_cols[0])[abl_i] = abl_out.pos;
    ((float2 *) A.out_cols[1])[abl_i] = abl_out.dir;
    ((float2 *) A.out_cols[2])[abl_i] = abl_out.steer;
    ((int *) A.out_cols[3])[abl_i] = abl_out.life;
}
#ifndef ABL_PERSIST
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ens_pred_avoid(const __grid_constant__ abl_ens_launch A) {
    abl_ens_body_pred_avoid(A, blockIdx.x, A.timestep);
}
static int abl_launch_ens_pred_avoid(const abl_ens_launch *L, cudaStream_t abl_stream) {
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (L->n + abl_block - 1) / abl_block;
    abl_kernel_ens_pred_avoid<<<abl_grid, abl_block, L->smem, abl_stream>>>(*L);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
#ifndef ABL_PERSIST
static double abl_radius_pred_avoid(const void *abl_gp) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    return (double) (abl_G.SAME_SPECIES_AVOIDANCE_RADIUS);
}
#endif

__device__ static void pred_move(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Predator* in, Predator* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    float2 agent_position = in->pos;
    float2 agent_velocity = in->dir;
    float2 agent_steer = in->steer;
    agent_velocity = float2_add(agent_velocity, agent_steer);
    double current_speed = length_float2(agent_velocity);
    if ((current_speed > 1.0)) {
        agent_velocity = normalize_float2(agent_velocity);
    }
    agent_position = float2_add(agent_position, float2_mul_scalar(float2_mul_scalar(float2_mul_scalar(agent_velocity, abl_G.DELTA_TIME), abl_G.PRED_SPEED_ADVANTAGE), abl_G.SPACE_MULT));
    agent_position = boundPosition(abl_G, abl_R, agent_position);
    out->pos = agent_position;
    out->dir = agent_velocity;
    out->life = (in->life - 1);
}

#ifndef ABL_PERSIST
struct abl_kargs_pred_move {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Predator in, out;
    abl_near_view NB;
    uint8_t *removed;
    uint8_t *child_flag;
    void *child_cols[ABL_MAX_MEMBERS];
    uint64_t seed;
    long timestep;
    int step_index;
    uint32_t skip_store;
    unsigned long long *serial_rng;
};
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_pred_move(const __grid_constant__ abl_kargs_pred_move A) {
    const long abl_t = (long) blockIdx.x * blockDim.x + threadIdx.x;
    if (abl_t >= A.n) return;
    const long abl_i = A.visit ? (long) A.visit[abl_t] : abl_t;
    abl::step_ctx abl_K;
    abl_K.R.init(A.seed, (uint32_t) abl_i, (uint32_t) A.step_index, (uint64_t) A.timestep);
    abl_K.R.xs = A.serial_rng;
    abl_K.self = abl_i;
    abl_K.removed = 0;
    abl_K.added = 0;
    abl_K.child_cols = A.child_cols;
    abl_K.near_col = -1;
    Predator abl_in, abl_out;
    abl_in.pos = A.in.pos[abl_i];
    abl_in.dir = A.in.dir[abl_i];
    abl_in.steer = A.in.steer[abl_i];
    abl_in.life = A.in.life[abl_i];
    abl_out = abl_in;
    pred_move(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.pos[abl_i] = abl_out.pos;
    A.out.dir[abl_i] = abl_out.dir;
    A.out.steer[abl_i] = abl_out.steer;
    A.out.life[abl_i] = abl_out.life;
}
static int abl_launch_pred_move(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_pred_move A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.pos = (float2 *) L->in_cols[0];
    A.out.pos = (float2 *) L->out_cols[0];
    A.in.dir = (float2 *) L->in_cols[1];
    A.out.dir = (float2 *) L->out_cols[1];
    A.in.steer = (float2 *) L->in_cols[2];
    A.out.steer = (float2 *) L->out_cols[2];
    A.in.life = (int *) L->in_cols[3];
    A.out.life = (int *) L->out_cols[3];
    A.NB = L->near;
    A.removed = L->removed;
    A.child_flag = L->child_flag;
    for (int k = 0; k < ABL_MAX_MEMBERS; k++) A.child_cols[k] = L->child_cols[k];
    A.seed = L->seed;
    A.timestep = L->timestep;
    A.step_index = L->step_index;
    A.skip_store = L->skip_store;
    A.serial_rng = L->serial_rng;
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (A.n + abl_block - 1) / abl_block;
    abl_kernel_pred_move<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
__device__ __forceinline__ void abl_ens_body_pred_move(const abl_ens_launch &A, long abl_vb, long abl_ts) {
    const long abl_t = abl_vb * blockDim.x + threadIdx.x;
    if (abl_t >= A.n) return;
    const long abl_i = A.visit_order ? (long) A.visit_order[abl_t] : abl_t;
    const int abl_r = A.replica[abl_i];
    const abl_globals &abl_Gr = ((const abl_globals *) A.globals)[abl_r];
    abl::step_ctx abl_K;
    abl_K.R.init(A.seeds[abl_r], (uint32_t) (abl_i - A.agent_base[abl_r]), (uint32_t) A.step_index, (uint64_t) abl_ts);
    abl_K.self = abl_i;
    abl_K.removed = 0;
    abl_K.added = 0;
    abl_K.child_cols = nullptr;
    abl_K.near_col = -1;
    Predator abl_in, abl_out;
    abl_in.pos = ((const float2 *) A.in_cols[0])[abl_i];
    abl_in.dir = ((const float2 *) A.in_cols[1])[abl_i];
    abl_in.steer = ((const float2 *) A.in_cols[2])[abl_i];
    abl_in.life = ((const int *) A.in_cols[3])[abl_i];
    abl_out.pos = abl_in.pos;
    abl_out.dir = abl_in.dir;
    abl_out.steer = abl_in.steer;
    abl_out.life = abl_in.life;
    pred_move(abl_Gr, A.views[abl_r], abl_K, &abl_in, &abl_out);
    ((float2 *) A.out_cols[0])[abl_i] = abl_out.pos;
    ((float2 *) A.out_cols[1])[abl_i] = abl_out.dir;
    ((float2 *) A.out_cols[2])[abl_i] = abl_out.steer;
    ((int *) A.out_cols[3])[abl_i] = abl_out.life;
}
#ifndef ABL_PERSIST
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ens_pred_move(const __grid_constant__ abl_ens_launch A) {
    abl_ens_body_pred_move(A, blockIdx.x, A.timestep);
}
static int abl_launch_ens_pred_move(const abl_ens_launch *L, cudaStream_t abl_stream) {
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (L->n + abl_block - 1) / abl_block;
    abl_kernel_ens_pred_move<<<abl_grid, abl_block, L->smem, abl_stream>>>(*L);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif

__device__ static void pred_eat_or_starve(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Predator* in, Predator* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    int pred_life = in->life;
    {
        const abl::near_query<2> abl_q7(abl_NB, (double) in->pos.x, (double) in->pos.y, 0.0, abl_K.self);
        abl::near_cursor<2> abl_c7(abl_NB, abl_q7);
        auto abl_exact7 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) abl_NB.cols[0])[abl_s];
            return !(dist_float2(abl_p, in->pos) > abl_G.PRED_KILL_DISTANCE);
        };
        while (abl_c7.fill(abl_q7, abl_exact7)) {
            int abl_pslot7 = abl_c7.slot(0);
            Prey abl_pnx7;
            for (int abl_k = 0; abl_k < abl_c7.cnt; ++abl_k) {
                const int abl_slot7 = abl_pslot7;
                Prey abl_nx7 = abl_pnx7;
                if (abl_k + 1 < abl_c7.cnt) {
                    abl_pslot7 = abl_c7.slot(abl_k + 1);
                }
                Prey* prey = &abl_nx7;
                {
                    pred_life += abl_G.GAIN_FROM_FOOD_PREDATOR;
                }
            }
        }
    }
    out->life = pred_life;
    if ((pred_life < 1)) abl_K.remove();
}

#ifndef ABL_PERSIST
struct abl_kargs_pred_eat_or_starve {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Predator in, out;
    abl_near_view NB;
    uint8_t *removed;
    uint8_t *child_flag;
    void *child_cols[ABL_MAX_MEMBERS];
    uint64_t seed;
    long timestep;
    int step_index;
    uint32_t skip_store;
    unsigned long long *serial_rng;
};
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_pred_eat_or_starve(const __grid_constant__ abl_kargs_pred_eat_or_starve A) {
    const long abl_t = (long) blockIdx.x * blockDim.x + threadIdx.x;
    if (abl_t >= A.n) return;
    const long abl_i = A.visit ? (long) A.visit[abl_t] : abl_t;
    abl::step_ctx abl_K;
    abl_K.R.init(A.seed, (uint32_t) abl_i, (uint32_t) A.step_index, (uint64_t) A.timestep);
    abl_K.R.xs = A.serial_rng;
    abl_K.self = abl_i;
    abl_K.removed = 0;
    abl_K.added = 0;
    abl_K.child_cols = A.child_cols;
    abl_K.near_col = -1;
    Predator abl_in, abl_out;
    abl_in.pos = A.in.pos[abl_i];
    abl_in.dir = A.in.dir[abl_i];
    abl_in.steer = A.in.steer[abl_i];
    abl_in.life = A.in.life[abl_i];
    abl_out = abl_in;
    pred_eat_or_starve(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.pos[abl_i] = abl_out.pos;
    A.out.dir[abl_i] = abl_out.dir;
    A.out.steer[abl_i] = abl_out.steer;
    A.out.life[abl_i] = abl_out.life;
    A.removed[abl_i] = (uint8_t) abl_K.removed;
}
static int abl_launch_pred_eat_or_starve(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_pred_eat_or_starve A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.pos = (float2 *) L->in_cols[0];
    A.out.pos = (float2 *) L->out_cols[0];
    A.in.dir = (float2 *) L->in_cols[1];
    A.out.dir = (float2 *) L->out_cols[1];
    A.in.steer = (float2 *) L->in_cols[2];
    A.out.steer = (float2 *) L->out_cols[2];
    A.in.life = (int *) L->in_cols[3];
    A.out.life = (int *) L->out_cols[3];
    A.NB = L->near;
    A.removed = L->removed;
    A.child_flag = L->child_flag;
    for (int k = 0; k < ABL_MAX_MEMBERS; k++) A.child_cols[k] = L->child_cols[k];
    A.seed = L->seed;
    A.timestep = L->timestep;
    A.step_index = L->step_index;
    A.skip_store = L->skip_store;
    A.serial_rng = L->serial_rng;
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (A.n + abl_block - 1) / abl_block;
    abl_kernel_pred_eat_or_starve<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
#ifndef ABL_PERSIST
static double abl_radius_pred_eat_or_starve(const void *abl_gp) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    return (double) (abl_G.PRED_KILL_DISTANCE);
}
#endif

__device__ static void pred_reproduction(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Predator* in, Predator* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    if ((random_3(abl_G, abl_R, 1.0) < abl_G.REPRODUCE_PREDATOR_PROB)) {
        abl_add_Predator(abl_K, ([&]() { Predator abl_a; abl_a.pos = in->pos; abl_a.dir = float2_mul_scalar(in->dir, -1.0); abl_a.steer = float2_mul_scalar(in->steer, -1.0); abl_a.life = (in->life / 2); return abl_a; }()));
        out->life = (in->life / 2);
    }
}

#ifndef ABL_PERSIST
struct abl_kargs_pred_reproduction {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Predator in, out;
    abl_near_view NB;
    uint8_t *removed;
    uint8_t *child_flag;
    void *child_cols[ABL_MAX_MEMBERS];
    uint64_t seed;
    long timestep;
    int step_index;
    uint32_t skip_store;
    unsigned long long *serial_rng;
};
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_pred_reproduction(const __grid_constant__ abl_kargs_pred_reproduction A) {
    const long abl_t = (long) blockIdx.x * blockDim.x + threadIdx.x;
    if (abl_t >= A.n) return;
    const long abl_i = A.visit ? (long) A.visit[abl_t] : abl_t;
    abl::step_ctx abl_K;
    abl_K.R.init(A.seed, (uint32_t) abl_i, (uint32_t) A.step_index, (uint64_t) A.timestep);
    abl_K.R.xs = A.serial_rng;
    abl_K.self = abl_i;
    abl_K.removed = 0;
    abl_K.added = 0;
    abl_K.child_cols = A.child_cols;
    abl_K.near_col = -1;
    Predator abl_in, abl_out;
    abl_in.pos = A.in.pos[abl_i];
    abl_in.dir = A.in.dir[abl_i];
    abl_in.steer = A.in.steer[abl_i];
    abl_in.life = A.in.life[abl_i];
    abl_out = abl_in;
    pred_reproduction(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.pos[abl_i] = abl_out.pos;
    A.out.dir[abl_i] = abl_out.dir;
    A.out.steer[abl_i] = abl_out.steer;
    A.out.life[abl_i] = abl_out.life;
    A.child_flag[abl_i] = (uint8_t) abl_K.added;
}
static int abl_launch_pred_reproduction(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_pred_reproduction A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.pos = (float2 *) L->in_cols[0];
    A.out.pos = (float2 *) L->out_cols[0];
    A.in.dir = (float2 *) L->in_cols[1];
    A.out.dir = (float2 *) L->out_cols[1];
    A.in.steer = (float2 *) L->in_cols[2];
    A.out.steer = (float2 *) L->out_cols[2];
    A.in.life = (int *) L->in_cols[3];
    A.out.life = (int *) L->out_cols[3];
    A.NB = L->near;
    A.removed = L->removed;
    A.child_flag = L->child_flag;
    for (int k = 0; k < ABL_MAX_MEMBERS; k++) A.child_cols[k] = L->child_cols[k];
    A.seed = L->seed;
    A.timestep = L->timestep;
    A.step_index = L->step_index;
    A.skip_store = L->skip_store;
    A.serial_rng = L->serial_rng;
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (A.n + abl_block - 1) / abl_block;
    abl_kernel_pred_reproduction<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif

__device__ static void grass_eaten(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Grass* in, Grass* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    double closest_prey = abl_G.GRASS_EAT_DISTANCE;
    bool eaten = false;
    {
        const abl::near_query<2> abl_q8(abl_NB, (double) in->pos.x, (double) in->pos.y, 0.0, abl_K.self);
        abl::near_list_cursor<2> abl_c8(abl_NB, abl_q8, abl_K);
        auto abl_exact8 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) abl_NB.cols[0])[abl_s];
            return !(dist_float2(abl_p, in->pos) > abl_G.GRASS_EAT_DISTANCE);
        };
        while (abl_c8.fill(abl_q8, abl_exact8)) {
            int abl_pslot8 = abl_c8.slot(0);
            Prey abl_pnx8;
            abl_pnx8.pos = ((const float2 *) abl_NB.cols[0])[abl_pslot8];
            for (int abl_k = 0; abl_k < abl_c8.cnt; ++abl_k) {
                const int abl_slot8 = abl_pslot8;
                Prey abl_nx8 = abl_pnx8;
                if (abl_k + 1 < abl_c8.cnt) {
                    abl_pslot8 = abl_c8.slot(abl_k + 1);
                    abl_pnx8.pos = ((const float2 *) abl_NB.cols[0])[abl_pslot8];
                }
                Prey* prey = &abl_nx8;
                {
                    double distance = length_float2(float2_sub(in->pos, prey->pos));
                    if (((distance < closest_prey) && in->avail)) {
                        closest_prey = distance;
                        eaten = true;
                    }
                }
            }
        }
    }
    if (eaten) {
        out->dead_cycles = 0;
        out->avail = false;
    }
}

#ifndef ABL_PERSIST
struct abl_kargs_grass_eaten {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Grass in, out;
    abl_near_view NB;
    uint8_t *removed;
    uint8_t *child_flag;
    void *child_cols[ABL_MAX_MEMBERS];
    uint64_t seed;
    long timestep;
    int step_index;
    uint32_t skip_store;
    unsigned long long *serial_rng;
};
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_grass_eaten(const __grid_constant__ abl_kargs_grass_eaten A) {
    int abl_j;
    {
        const abl_globals &abl_G = A.G;
        const long abl_t1 = (long) blockIdx.x * blockDim.x + threadIdx.x;
        const bool abl_has = abl_t1 < A.n;
        const long abl_i1 = abl_has ? (A.visit ? (long) A.visit[abl_t1] : abl_t1) : 0;
        const float2 abl_p1 = abl_has ? A.in.pos[abl_i1] : float2{};
        const abl::near_query<2> abl_q0(A.NB, (double) abl_p1.x, (double) abl_p1.y, 0.0, abl_has ? abl_i1 : -1);
        auto abl_x0 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) A.NB.cols[0])[abl_s];
            return !(dist_float2(abl_p, abl_p1) > abl_G.GRASS_EAT_DISTANCE);
        };
        abl_j = abl::presort_block<2>(A.NB, abl_has, abl_q0, abl_x0);
    }
    const long abl_t = (long) blockIdx.x * blockDim.x + abl_j;
    if (abl_t >= A.n) return;
    const long abl_i = A.visit ? (long) A.visit[abl_t] : abl_t;
    abl::step_ctx abl_K;
    abl_K.R.init(A.seed, (uint32_t) abl_i, (uint32_t) A.step_index, (uint64_t) A.timestep);
    abl_K.R.xs = A.serial_rng;
    abl_K.self = abl_i;
    abl_K.removed = 0;
    abl_K.added = 0;
    abl_K.child_cols = A.child_cols;
    abl_K.near_col = abl_j;
    Grass abl_in, abl_out;
    abl_in.pos = A.in.pos[abl_i];
    abl_in.dead_cycles = A.in.dead_cycles[abl_i];
    abl_in.avail = A.in.avail[abl_i];
    abl_out = abl_in;
    grass_eaten(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.pos[abl_i] = abl_out.pos;
    A.out.dead_cycles[abl_i] = abl_out.dead_cycles;
    A.out.avail[abl_i] = abl_out.avail;
}
static int abl_launch_grass_eaten(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_grass_eaten A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.pos = (float2 *) L->in_cols[0];
    A.out.pos = (float2 *) L->out_cols[0];
    A.in.dead_cycles = (int *) L->in_cols[1];
    A.out.dead_cycles = (int *) L->out_cols[1];
    A.in.avail = (bool *) L->in_cols[2];
    A.out.avail = (bool *) L->out_cols[2];
    A.NB = L->near;
    A.removed = L->removed;
    A.child_flag = L->child_flag;
    for (int k = 0; k < ABL_MAX_MEMBERS; k++) A.child_cols[k] = L->child_cols[k];
    A.seed = L->seed;
    A.timestep = L->timestep;
    A.step_index = L->step_index;
    A.skip_store = L->skip_store;
    A.serial_rng = L->serial_rng;
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (A.n + abl_block - 1) / abl_block;
    abl_kernel_grass_eaten<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
__device__ __forceinline__ void abl_ens_body_grass_eaten(const abl_ens_launch &A, long abl_vb, long abl_ts) {
    int abl_j;
    {
        const long abl_t1 = abl_vb * blockDim.x + threadIdx.x;
        const bool abl_has = abl_t1 < A.n;
        const long abl_i1 = abl_has ? (A.visit_order ? (long) A.visit_order[abl_t1] : abl_t1) : 0;
        const int abl_r1 = abl_has ? A.replica[abl_i1] : 0;
        const abl_globals &abl_G = ((const abl_globals *) A.globals)[abl_r1];
        const abl_near_view &abl_V1 = A.views[abl_r1];
        const float2 abl_p1 = abl_has ? ((const float2 *) A.in_cols[0])[abl_i1] : float2{};
        const abl::near_query<2> abl_q0(abl_V1, (double) abl_p1.x, (double) abl_p1.y, 0.0, abl_has ? abl_i1 : -1);
        auto abl_x0 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) abl_V1.cols[0])[abl_s];
            return !(dist_float2(abl_p, abl_p1) > abl_G.GRASS_EAT_DISTANCE);
        };
        abl_j = abl::presort_block<2>(abl_V1, abl_has, abl_q0, abl_x0);
    }
    const long abl_t = abl_vb * blockDim.x + abl_j;
    if (abl_t >= A.n) return;
    const long abl_i = A.visit_order ? (long) A.visit_order[abl_t] : abl_t;
    const int abl_r = A.replica[abl_i];
    const abl_globals &abl_Gr = ((const abl_globals *) A.globals)[abl_r];
    abl::step_ctx abl_K;
    abl_K.R.init(A.seeds[abl_r], (uint32_t) (abl_i - A.agent_base[abl_r]), (uint32_t) A.step_index, (uint64_t) abl_ts);
    abl_K.self = abl_i;
    abl_K.removed = 0;
    abl_K.added = 0;
    abl_K.child_cols = nullptr;
    abl_K.near_col = abl_j;
    Grass abl_in, abl_out;
    abl_in.pos = ((const float2 *) A.in_cols[0])[abl_i];
    abl_in.dead_cycles = ((const int *) A.in_cols[1])[abl_i];
    abl_in.avail = ((const bool *) A.in_cols[2])[abl_i];
    abl_out.pos = abl_in.pos;
    abl_out.dead_cycles = abl_in.dead_cycles;
    abl_out.avail = abl_in.avail;
    grass_eaten(abl_Gr, A.views[abl_r], abl_K, &abl_in, &abl_out);
    ((float2 *) A.out_cols[0])[abl_i] = abl_out.pos;
    ((int *) A.out_cols[1])[abl_i] = abl_out.dead_cycles;
    ((bool *) A.out_cols[2])[abl_i] = abl_out.avail;
}
#ifndef ABL_PERSIST
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ens_grass_eaten(const __grid_constant__ abl_ens_launch A) {
    abl_ens_body_grass_eaten(A, blockIdx.x, A.timestep);
}
static int abl_launch_ens_grass_eaten(const abl_ens_launch *L, cudaStream_t abl_stream) {
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (L->n + abl_block - 1) / abl_block;
    abl_kernel_ens_grass_eaten<<<abl_grid, abl_block, L->smem, abl_stream>>>(*L);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
#ifndef ABL_PERSIST
static double abl_radius_grass_eaten(const void *abl_gp) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    return (double) (abl_G.GRASS_EAT_DISTANCE);
}
#endif

__device__ static void grass_growth(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Grass* in, Grass* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    if ((in->dead_cycles == abl_G.GRASS_REGROW_CYCLES)) {
        int cycle_start = 0;
        out->dead_cycles = cycle_start;
        out->avail = true;
    }
    if ((!in->avail)) out->dead_cycles = (in->dead_cycles + 1);
}

#ifndef ABL_PERSIST
struct abl_kargs_grass_growth {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Grass in, out;
    abl_near_view NB;
    uint8_t *removed;
    uint8_t *child_flag;
    void *child_cols[ABL_MAX_MEMBERS];
    uint64_t seed;
    long timestep;
    int step_index;
    uint32_t skip_store;
    unsigned long long *serial_rng;
};
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_grass_growth(const __grid_constant__ abl_kargs_grass_growth A) {
    const long abl_t = (long) blockIdx.x * blockDim.x + threadIdx.x;
    if (abl_t >= A.n) return;
    const long abl_i = A.visit ? (long) A.visit[abl_t] : abl_t;
    abl::step_ctx abl_K;
    abl_K.R.init(A.seed, (uint32_t) abl_i, (uint32_t) A.step_index, (uint64_t) A.timestep);
    abl_K.R.xs = A.serial_rng;
    abl_K.self = abl_i;
    abl_K.removed = 0;
    abl_K.added = 0;
    abl_K.child_cols = A.child_cols;
    abl_K.near_col = -1;
    Grass abl_in, abl_out;
    abl_in.pos = A.in.pos[abl_i];
    abl_in.dead_cycles = A.in.dead_cycles[abl_i];
    abl_in.avail = A.in.avail[abl_i];
    abl_out = abl_in;
    grass_growth(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.pos[abl_i] = abl_out.pos;
    A.out.dead_cycles[abl_i] = abl_out.dead_cycles;
    A.out.avail[abl_i] = abl_out.avail;
}
static int abl_launch_grass_growth(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_grass_growth A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.pos = (float2 *) L->in_cols[0];
    A.out.pos = (float2 *) L->out_cols[0];
    A.in.dead_cycles = (int *) L->in_cols[1];
    A.out.dead_cycles = (int *) L->out_cols[1];
    A.in.avail = (bool *) L->in_cols[2];
    A.out.avail = (bool *) L->out_cols[2];
    A.NB = L->near;
    A.removed = L->removed;
    A.child_flag = L->child_flag;
    for (int k = 0; k < ABL_MAX_MEMBERS; k++) A.child_cols[k] = L->child_cols[k];
    A.seed = L->seed;
    A.timestep = L->timestep;
    A.step_index = L->step_index;
    A.skip_store = L->skip_store;
    A.serial_rng = L->serial_rng;
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (A.n + abl_block - 1) / abl_block;
    abl_kernel_grass_growth<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
__device__ __forceinline__ void abl_ens_body_grass_growth(const abl_ens_launch &A, long abl_vb, long abl_ts) {
    const long abl_t = abl_vb * blockDim.x + threadIdx.x;
    if (abl_t >= A.n) return;
    const long abl_i = A.visit_order ? (long) A.visit_order[abl_t] : abl_t;
    const int abl_r = A.replica[abl_i];
    const abl_globals &abl_Gr = ((const abl_globals *) A.globals)[abl_r];
    abl::step_ctx abl_K;
    abl_K.R.init(A.seeds[abl_r], (uint32_t) (abl_i - A.agent_base[abl_r]), (uint32_t) A.step_index, (uint64_t) abl_ts);
    abl_K.self = abl_i;
    abl_K.removed = 0;
    abl_K.added = 0;
    abl_K.child_cols = nullptr;
    abl_K.near_col = -1;
    Grass abl_in, abl_out;
    abl_in.pos = ((const float2 *) A.in_cols[0])[abl_i];
    abl_in.dead_cycles = ((const int *) A.in_cols[1])[abl_i];
    abl_in.avail = ((const bool *) A.in_cols[2])[abl_i];
    abl_out.pos = abl_in.pos;
    abl_out.dead_cycles = abl_in.dead_cycles;
    abl_out.avail = abl_in.avail;
    grass_growth(abl_Gr, A.views[abl_r], abl_K, &abl_in, &abl_out);
    ((float2 *) A.out_cols[0])[abl_i] = abl_out.pos;
    ((int *) A.out_cols[1])[abl_i] = abl_out.dead_cycles;
    ((bool *) A.out_cols[2])[abl_i] = abl_out.avail;
}
#ifndef ABL_PERSIST
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ens_grass_growth(const __grid_constant__ abl_ens_launch A) {
    abl_ens_body_grass_growth(A, blockIdx.x, A.timestep);
}
static int abl_launch_ens_grass_growth(const abl_ens_launch *L, cudaStream_t abl_stream) {
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (L->n + abl_block - 1) / abl_block;
    abl_kernel_ens_grass_growth<<<abl_grid, abl_block, L->smem, abl_stream>>>(*L);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif

static int abl_seq_gather_stats(abl_ctx *abl_C, const void *abl_gp) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R_host;
    abl::rng &abl_R = abl_R_host;
    (void) abl_G; (void) abl_R;
    int num_prey = abl_seq_count(abl_C, 1);
    int num_predator = abl_seq_count(abl_C, 0);
    int num_avail_grass = abl_seq_sum<int>(abl_C, 2, 2);
    double exec_time = abl_seq_exec_time(abl_C);
    abl_log_csv(abl_C, "%d,%d,%d,%f\n", num_prey, num_predator, num_avail_grass, exec_time);
    return ABL_OK;
}

#ifndef ABL_PERSIST
static const abl_member_desc abl_members_Predator[] = {
    {"pos", ABL_T_FLOAT2, 2, 8, 1},
    {"dir", ABL_T_FLOAT2, 2, 8, 0},
    {"steer", ABL_T_FLOAT2, 2, 8, 0},
    {"life", ABL_T_INT, 1, 4, 0},
};
static const abl_member_desc abl_members_Prey[] = {
    {"pos", ABL_T_FLOAT2, 2, 8, 1},
    {"dir", ABL_T_FLOAT2, 2, 8, 0},
    {"steer", ABL_T_FLOAT2, 2, 8, 0},
    {"life", ABL_T_INT, 1, 4, 0},
};
static const abl_member_desc abl_members_Grass[] = {
    {"pos", ABL_T_FLOAT2, 2, 8, 1},
    {"dead_cycles", ABL_T_INT, 1, 4, 0},
    {"avail", ABL_T_BOOL, 1, 1, 0},
};
static const abl_agent_desc abl_agents[] = {
    {"Predator", 4, abl_members_Predator, 0, 2},
    {"Prey", 4, abl_members_Prey, 0, 2},
    {"Grass", 3, abl_members_Grass, 0, 2},
};
static const abl_global_desc abl_global_table[] = {
    {"PI", ABL_T_FLOAT, offsetof(abl_globals, PI)},
    {"SPACE_MULT", ABL_T_FLOAT, offsetof(abl_globals, SPACE_MULT)},
    {"REPRODUCE_PREY_PROB", ABL_T_FLOAT, offsetof(abl_globals, REPRODUCE_PREY_PROB)},
    {"REPRODUCE_PREDATOR_PROB", ABL_T_FLOAT, offsetof(abl_globals, REPRODUCE_PREDATOR_PROB)},
    {"GAIN_FROM_FOOD_PREDATOR", ABL_T_INT, offsetof(abl_globals, GAIN_FROM_FOOD_PREDATOR)},
    {"GAIN_FROM_FOOD_PREY", ABL_T_INT, offsetof(abl_globals, GAIN_FROM_FOOD_PREY)},
    {"GRASS_REGROW_CYCLES", ABL_T_INT, offsetof(abl_globals, GRASS_REGROW_CYCLES)},
    {"PRED_PREY_INTERACTION_RADIUS", ABL_T_FLOAT, offsetof(abl_globals, PRED_PREY_INTERACTION_RADIUS)},
    {"PREY_GROUP_COHESION_RADIUS", ABL_T_FLOAT, offsetof(abl_globals, PREY_GROUP_COHESION_RADIUS)},
    {"SAME_SPECIES_AVOIDANCE_RADIUS", ABL_T_FLOAT, offsetof(abl_globals, SAME_SPECIES_AVOIDANCE_RADIUS)},
    {"GRASS_EAT_DISTANCE", ABL_T_FLOAT, offsetof(abl_globals, GRASS_EAT_DISTANCE)},
    {"PRED_KILL_DISTANCE", ABL_T_FLOAT, offsetof(abl_globals, PRED_KILL_DISTANCE)},
    {"DELTA_TIME", ABL_T_FLOAT, offsetof(abl_globals, DELTA_TIME)},
    {"PRED_SPEED_ADVANTAGE", ABL_T_FLOAT, offsetof(abl_globals, PRED_SPEED_ADVANTAGE)},
    {"prey_fraction", ABL_T_FLOAT, offsetof(abl_globals, prey_fraction)},
    {"predator_fraction", ABL_T_FLOAT, offsetof(abl_globals, predator_fraction)},
    {"agent_density", ABL_T_FLOAT, offsetof(abl_globals, agent_density)},
    {"num_agents", ABL_T_INT, offsetof(abl_globals, num_agents)},
    {"num_timesteps", ABL_T_INT, offsetof(abl_globals, num_timesteps)},
    {"env_size", ABL_T_FLOAT, offsetof(abl_globals, env_size)},
    {nullptr, 0, 0}
};
static void abl_env_bounds(const void *abl_gp, double *abl_min, double *abl_max) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    float2 abl_lo = float2_fill(0);
    float2 abl_hi = float2_fill(abl_G.env_size);
    abl_min[0] = abl_lo.x; abl_min[1] = abl_lo.y; abl_min[2] = 0;
    abl_max[0] = abl_hi.x; abl_max[1] = abl_hi.y; abl_max[2] = 0;
}
static const abl_step_desc abl_steps[] = {
    {"prey_avoid_pred", 1, 0, 1, abl_radius_prey_avoid_pred, 1u, 4u, abl_launch_prey_avoid_pred, 0, -1, 1, abl_launch_ens_prey_avoid_pred, 0, 1, 4u, 1},
    {"prey_flock", 1, 1, 1, abl_radius_prey_flock, 1u, 4u, abl_launch_prey_flock, 0, -1, 1, abl_launch_ens_prey_flock, 0, 1, 4u, 1},
    {"prey_move", 1, -1, 1, nullptr, 0u, 11u, abl_launch_prey_move, 0, -1, 1, abl_launch_ens_prey_move, 0, 0, 11u, 0},
    {"prey_eaten", 1, 0, 1, abl_radius_prey_eaten, 1u, 0u, abl_launch_prey_eaten, 1, -1, 1, nullptr, 0, 1, 0u, 1},
    {"prey_eat_or_starve", 1, 2, 0, abl_radius_prey_eat_or_starve, 5u, 8u, abl_launch_prey_eat_or_starve, 1, -1, 1, nullptr, 0, 0, 8u, 1},
    {"prey_reproduction", 1, -1, 1, nullptr, 0u, 0u, abl_launch_prey_reproduction, 0, 1, 1, nullptr, 1, 0, 8u, 0},
    {"pred_follow_prey", 0, 1, 1, abl_radius_pred_follow_prey, 1u, 4u, abl_launch_pred_follow_prey, 0, -1, 1, abl_launch_ens_pred_follow_prey, 0, 1, 4u, 1},
    {"pred_avoid", 0, 0, 1, abl_radius_pred_avoid, 1u, 4u, abl_launch_pred_avoid, 0, -1, 1, abl_launch_ens_pred_avoid, 0, 1, 4u, 1},
    {"pred_move", 0, -1, 1, nullptr, 0u, 11u, abl_launch_pred_move, 0, -1, 1, abl_launch_ens_pred_move, 0, 0, 11u, 0},
    {"pred_eat_or_starve", 0, 1, 0, abl_radius_pred_eat_or_starve, 1u, 8u, abl_launch_pred_eat_or_starve, 1, -1, 1, nullptr, 0, 0, 8u, 1},
    {"pred_reproduction", 0, -1, 1, nullptr, 0u, 0u, abl_launch_pred_reproduction, 0, 0, 1, nullptr, 1, 0, 8u, 0},
    {"grass_eaten", 2, 1, 1, abl_radius_grass_eaten, 1u, 0u, abl_launch_grass_eaten, 0, -1, 1, abl_launch_ens_grass_eaten, 0, 1, 6u, 1},
    {"grass_growth", 2, -1, 1, nullptr, 0u, 0u, abl_launch_grass_growth, 0, -1, 1, abl_launch_ens_grass_growth, 0, 0, 6u, 0},
};
static const abl_step_desc abl_steps_ordered[] = {
    abl_steps[6],
    abl_steps[0],
    abl_steps[1],
    abl_steps[7],
    abl_steps[2],
    abl_steps[8],
    abl_steps[4],
    abl_steps[9],
    abl_steps[11],
    abl_steps[3],
    abl_steps[10],
    abl_steps[5],
    abl_steps[12],
    {nullptr, 0, -1, 0, nullptr, 0u, 0u, nullptr, 0, -1, 0, nullptr, 0}
};
extern const abl_model_desc abl_desc = {
    "predator_prey", 3, abl_agents, 13, abl_steps_ordered, sizeof(abl_globals), &abl_globals_default, 20, abl_global_table, 2, abl_env_bounds, nullptr, 0, abl_seq_gather_stats, nullptr
};
static void abl_check(int r, const char *what) {
    if (r != ABL_OK) {
        std::fprintf(stderr, "%s failed: %s\n", what, abl_strerror(r));
        std::exit(1);
    }
}
static void abl_simulate(int abl_timesteps) {
    abl_ctx *ctx = nullptr;
    abl_check(abl_create(&abl_desc, 0, &ctx), "abl_create");
    abl_check(abl_set_globals(ctx, &abl_G, sizeof abl_G), "abl_set_globals");
    {
        size_t n = agents.agents_Predator.len;
        const Predator *aos = (const Predator *) agents.agents_Predator.values;
        float2 *c0 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c0[i] = aos[i].pos;
        float2 *c1 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c1[i] = aos[i].dir;
        float2 *c2 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c2[i] = aos[i].steer;
        int *c3 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c3[i] = aos[i].life;
        const void *cols[] = {c0, c1, c2, c3};
        abl_check(abl_upload(ctx, 0, cols, n), "abl_upload");
        std::free(c0);
        std::free(c1);
        std::free(c2);
        std::free(c3);
    }
    {
        size_t n = agents.agents_Prey.len;
        const Prey *aos = (const Prey *) agents.agents_Prey.values;
        float2 *c0 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c0[i] = aos[i].pos;
        float2 *c1 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c1[i] = aos[i].dir;
        float2 *c2 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c2[i] = aos[i].steer;
        int *c3 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c3[i] = aos[i].life;
        const void *cols[] = {c0, c1, c2, c3};
        abl_check(abl_upload(ctx, 1, cols, n), "abl_upload");
        std::free(c0);
        std::free(c1);
        std::free(c2);
        std::free(c3);
    }
    {
        size_t n = agents.agents_Grass.len;
        const Grass *aos = (const Grass *) agents.agents_Grass.values;
        float2 *c0 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c0[i] = aos[i].pos;
        int *c1 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c1[i] = aos[i].dead_cycles;
        bool *c2 = (bool *) std::malloc(sizeof(bool) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c2[i] = aos[i].avail;
        const void *cols[] = {c0, c1, c2};
        abl_check(abl_upload(ctx, 2, cols, n), "abl_upload");
        std::free(c0);
        std::free(c1);
        std::free(c2);
    }
    #ifdef ABL_SERIAL_RANDOM
    uint64_t abl_xs[2];
    abl_host_rng_get(abl_xs);
    abl_check(abl_set_serial_random(ctx, abl_xs), "abl_set_serial_random");
    #endif
    abl_check(abl_run(ctx, abl_timesteps), "abl_run");
    #ifdef ABL_SERIAL_RANDOM
    abl_check(abl_get_serial_random(ctx, abl_xs), "abl_get_serial_random");
    abl_host_rng_set(abl_xs);
    #endif
    {
        size_t n = 0;
        abl_check(abl_count(ctx, 0, &n), "abl_count");
        float2 *c0 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        float2 *c1 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        float2 *c2 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        int *c3 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        void *cols[] = {c0, c1, c2, c3};
        size_t cap = n;
        abl_check(abl_download(ctx, 0, cols, &cap), "abl_download");
        dyn_array_clean(&agents.agents_Predator);
        agents.agents_Predator = dyn_array_create_fixed(sizeof(Predator), n);
        Predator *aos = (Predator *) agents.agents_Predator.values;
        for (size_t i = 0; i < n; i++) {
            aos[i].pos = c0[i];
            aos[i].dir = c1[i];
            aos[i].steer = c2[i];
            aos[i].life = c3[i];
        }
        std::free(c0);
        std::free(c1);
        std::free(c2);
        std::free(c3);
    }
    {
        size_t n = 0;
        abl_check(abl_count(ctx, 1, &n), "abl_count");
        float2 *c0 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        float2 *c1 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        float2 *c2 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        int *c3 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        void *cols[] = {c0, c1, c2, c3};
        size_t cap = n;
        abl_check(abl_download(ctx, 1, cols, &cap), "abl_download");
        dyn_array_clean(&agents.agents_Prey);
        agents.agents_Prey = dyn_array_create_fixed(sizeof(Prey), n);
        Prey *aos = (Prey *) agents.agents_Prey.values;
        for (size_t i = 0; i < n; i++) {
            aos[i].pos = c0[i];
            aos[i].dir = c1[i];
            aos[i].steer = c2[i];
            aos[i].life = c3[i];
        }
        std::free(c0);
        std::free(c1);
        std::free(c2);
        std::free(c3);
    }
    {
        size_t n = 0;
        abl_check(abl_count(ctx, 2, &n), "abl_count");
        float2 *c0 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        int *c1 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        bool *c2 = (bool *) std::malloc(sizeof(bool) * (n ? n : 1));
        void *cols[] = {c0, c1, c2};
        size_t cap = n;
        abl_check(abl_download(ctx, 2, cols, &cap), "abl_download");
        dyn_array_clean(&agents.agents_Grass);
        agents.agents_Grass = dyn_array_create_fixed(sizeof(Grass), n);
        Grass *aos = (Grass *) agents.agents_Grass.values;
        for (size_t i = 0; i < n; i++) {
            aos[i].pos = c0[i];
            aos[i].dead_cycles = c1[i];
            aos[i].avail = c2[i];
        }
        std::free(c0);
        std::free(c1);
        std::free(c2);
    }
    size_t abl_log_len = 0;
    abl_log_text(ctx, nullptr, 0, &abl_log_len);
    if (abl_log_len > 0) {
        char *abl_log = (char *) std::malloc(abl_log_len + 1);
        abl_log_text(ctx, abl_log, abl_log_len + 1, nullptr);
        FILE *abl_f = std::fopen("log.csv", "w");
        if (abl_f) { std::fputs(abl_log, abl_f); std::fclose(abl_f); }
        std::free(abl_log);
    }
    abl_destroy(ctx);
}
static int abl_main() {
    int num_predators = (int) (abl_G.predator_fraction * (float) abl_G.num_agents);
    int num_prey = (int) (abl_G.prey_fraction * (float) abl_G.num_agents);
    int num_grass = ((abl_G.num_agents - num_predators) - num_prey);
    for (int i = 0, _var0 = num_grass; i < _var0; ++i) {
        *DYN_ARRAY_PLACE(&agents.agents_Grass, Grass) = ([&]() { Grass abl_a; abl_a.pos = random_4(abl_G, abl_R, float2_fill(abl_G.env_size)); abl_a.dead_cycles = 0; abl_a.avail = true; return abl_a; }());
    }
    for (int i = 0, _var1 = num_prey; i < _var1; ++i) {
        *DYN_ARRAY_PLACE(&agents.agents_Prey, Prey) = ([&]() { Prey abl_a; abl_a.pos = random_4(abl_G, abl_R, float2_fill(abl_G.env_size)); abl_a.dir = randomDirection(abl_G, abl_R); abl_a.steer = float2_fill(0); abl_a.life = (abl_G.GAIN_FROM_FOOD_PREY + randomInt_1(abl_G, abl_R, 10)); return abl_a; }());
    }
    for (int i = 0, _var2 = num_predators; i < _var2; ++i) {
        *DYN_ARRAY_PLACE(&agents.agents_Predator, Predator) = ([&]() { Predator abl_a; abl_a.pos = random_4(abl_G, abl_R, float2_fill(abl_G.env_size)); abl_a.dir = randomDirection(abl_G, abl_R); abl_a.steer = float2_fill(0); abl_a.life = (abl_G.GAIN_FROM_FOOD_PREDATOR + randomInt_1(abl_G, abl_R, 10)); return abl_a; }());
    }
    abl_simulate(abl_G.num_timesteps);
    save(&agents, agents_info, "agents.json", SAVE_JSON);
    return 0;
}
#else
#endif

}  // namespace abl_model_predator_prey

#ifndef ABL_PERSIST
extern "C" const abl_model_desc *abl_model_desc_predator_prey(void) {
    return &abl_model_predator_prey::abl_desc;
}
#endif

#if defined(ABL_STANDALONE_MAIN) && !defined(ABL_PERSIST)
extern "C" const abl_model_desc *const abl_builtin_models[] = {
    &abl_model_predator_prey::abl_desc, nullptr};
int main() { return abl_model_predator_prey::abl_main(); }
#endif
