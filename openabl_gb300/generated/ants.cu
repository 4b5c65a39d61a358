// Generated by OpenABL -b cuda (model "ants").
#include "abl_gen.cuh"

namespace abl_model_ants {

typedef double abl_float;
#include "abl_math.cuh"

typedef struct {
    float2 pos;
    float2 last_pos;
    double reward;
    double max_home;
    double max_food;
    bool hasFood;
} Ant;
static const type_info Ant_info[] = {
    { TYPE_FLOAT2, offsetof(Ant, pos), "pos", true },
    { TYPE_FLOAT2, offsetof(Ant, last_pos), "last_pos", false },
    { TYPE_FLOAT, offsetof(Ant, reward), "reward", false },
    { TYPE_FLOAT, offsetof(Ant, max_home), "max_home", false },
    { TYPE_FLOAT, offsetof(Ant, max_food), "max_food", false },
    { TYPE_BOOL, offsetof(Ant, hasFood), "hasFood", false },
    { TYPE_END, sizeof(Ant), NULL }
};

typedef struct {
    float2 pos;
    double food;
    double home;
} Pheromone;
static const type_info Pheromone_info[] = {
    { TYPE_FLOAT2, offsetof(Pheromone, pos), "pos", true },
    { TYPE_FLOAT, offsetof(Pheromone, food), "food", false },
    { TYPE_FLOAT, offsetof(Pheromone, home), "home", false },
    { TYPE_END, sizeof(Pheromone), NULL }
};

struct agent_struct {
    dyn_array agents_Ant;
    dyn_array agents_Ant_dbuf;
    dyn_array agents_Pheromone;
    dyn_array agents_Pheromone_dbuf;
};
static struct agent_struct agents;
static const agent_info agents_info[] = {
    { Ant_info, offsetof(struct agent_struct, agents_Ant), "Ant" },
    { Pheromone_info, offsetof(struct agent_struct, agents_Pheromone), "Pheromone" },
    { NULL, 0, NULL }
};

struct abl_globals {
    double PI;
    double SQRT2;
    double evaporationConstant;
    double initialReward;
    double cutDown;
    double momentumProbability;
    double randomActionProbability;
    double pheromone_radius;
    double ants_density;
    int num_agents;
    int num_timesteps;
    int num_ants;
    int env_size;
    int num_pheromones;
    double env_scale;
    float2 home_pos;
    float2 food_pos;
};
static const abl_globals abl_globals_default = {
    3.14159,
    1.41421,
    0.999,
    1.0,
    0.9,
    0.8,
    0.1,
    1.42,
    0.1,
    11000,
    100,
    1000,
    100,
    10000,
    1.0,
    {75.5, 75.5},
    {25.5, 25.5},
};
static abl_globals abl_G = abl_globals_default;
static abl::rng abl_R;  // unused on the host: main() draws from the host stream
struct abl_cols_Ant {
    float2 *pos;
    float2 *last_pos;
    double *reward;
    double *max_home;
    double *max_food;
    bool *hasFood;
};
struct abl_cols_Pheromone {
    float2 *pos;
    double *food;
    double *home;
};

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
__host__ __device__ static inline bool random_boolean(const abl_globals &abl_G, abl::rng &abl_R, double p) {
    double val = random_3(abl_G, abl_R, 1.0);
    if ((val < p)) return true; else return false;
}
__host__ __device__ static inline bool is_obstacle(const abl_globals &abl_G, abl::rng &abl_R, float2 pos) {
    double a2 = ((36.0 * abl_G.env_scale) * abl_G.env_scale);
    double b2 = ((1024.0 * abl_G.env_scale) * abl_G.env_scale);
    float2 C1 = float2_mul_scalar(float2_create(45.5, 25.5), abl_G.env_scale);
    float2 f1 = float2_sub(pos, C1);
    float2 s1 = float2_mul_scalar(f1, 0.707);
    if ((((((s1.x + s1.y) * (s1.x + s1.y)) / a2) + (((s1.x - s1.y) * (s1.x - s1.y)) / b2)) <= 1)) return true;
    float2 C2 = float2_mul_scalar(float2_create(35.5, 70.5), abl_G.env_scale);
    float2 f2 = float2_sub(pos, C2);
    float2 s2 = float2_mul_scalar(f2, 0.707);
    if ((((((s2.x + s2.y) * (s2.x + s2.y)) / a2) + (((s2.x - s2.y) * (s2.x - s2.y)) / b2)) <= 1)) return true;
    return false;
}
__host__ __device__ static inline bool is_home(const abl_globals &abl_G, abl::rng &abl_R, float2 ant_pos) {
    return (dist_float2(ant_pos, abl_G.home_pos) <= (1.1 * abl_G.env_scale));
}
__host__ __device__ static inline bool is_food(const abl_globals &abl_G, abl::rng &abl_R, float2 ant_pos) {
    return (dist_float2(ant_pos, abl_G.food_pos) <= (1.1 * abl_G.env_scale));
}
__host__ __device__ static inline float2 random_displacement(const abl_globals &abl_G, abl::rng &abl_R) {
    int dx = abl_random_int(abl_R, (-1), 1);
    int dy = abl_random_int(abl_R, (-1), 1);
    return float2_create(dx, dy);
}
__host__ __device__ static inline float2 default_move(const abl_globals &abl_G, abl::rng &abl_R, float2 pos, float2 last_pos) {
    if (random_boolean(abl_G, abl_R, abl_G.momentumProbability)) {
        return float2_add(pos, float2_sub(pos, last_pos));
    } else {
        return float2_add(pos, random_displacement(abl_G, abl_R));
    }
}
__host__ __device__ static inline float2 pheromone_move(const abl_globals &abl_G, abl::rng &abl_R, float2 pos, float2 max_pos) {
    if (random_boolean(abl_G, abl_R, abl_G.randomActionProbability)) {
        return float2_add(pos, random_displacement(abl_G, abl_R));
    } else {
        return max_pos;
    }
}
__device__ static void ant_deposit(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Ant* in, Ant* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    double home_max = 0.0;
    double food_max = 0.0;
    {
        const abl::near_query<2> abl_q1(abl_NB, (double) in->pos.x, (double) in->pos.y, 0.0, abl_K.self);
        abl::near_list_cursor<2> abl_c1(abl_NB, abl_q1, abl_K);
        auto abl_exact1 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) abl_NB.cols[0])[abl_s];
            return !(dist_float2(abl_p, in->pos) > abl_G.pheromone_radius);
        };
        while (abl_c1.fill(abl_q1, abl_exact1)) {
            int abl_pslot1 = abl_c1.slot(0);
            Pheromone abl_pnx1;
            abl_pnx1.food = ((const double *) abl_NB.cols[1])[abl_pslot1];
            abl_pnx1.home = ((const double *) abl_NB.cols[2])[abl_pslot1];
            for (int abl_k = 0; abl_k < abl_c1.cnt; ++abl_k) {
                const int abl_slot1 = abl_pslot1;
                Pheromone abl_nx1 = abl_pnx1;
                if (abl_k + 1 < abl_c1.cnt) {
                    abl_pslot1 = abl_c1.slot(abl_k + 1);
                    abl_pnx1.food = ((const double *) abl_NB.cols[1])[abl_pslot1];
                    abl_pnx1.home = ((const double *) abl_NB.cols[2])[abl_pslot1];
                }
                Pheromone* px = &abl_nx1;
                {
                    double K = 1.0;
                    double home_m = (((px->home * K) * abl_G.cutDown) + in->reward);
                    home_max = max(home_max, home_m);
                    double food_m = (((px->food * K) * abl_G.cutDown) + in->reward);
                    food_max = max(food_max, food_m);
                }
            }
        }
    }
    if (in->hasFood) out->max_food = food_max; else out->max_home = home_max;
    out->reward = 0;
}

#ifndef ABL_PERSIST
struct abl_kargs_ant_deposit {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Ant in, out;
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
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ant_deposit(const __grid_constant__ abl_kargs_ant_deposit A) {
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
            return !(dist_float2(abl_p, abl_p1) > abl_G.pheromone_radius);
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
    Ant abl_in, abl_out;
    abl_in.pos = A.in.pos[abl_i];
    abl_in.last_pos = A.in.last_pos[abl_i];
    abl_in.reward = A.in.reward[abl_i];
    abl_in.max_home = A.in.max_home[abl_i];
    abl_in.max_food = A.in.max_food[abl_i];
    abl_in.hasFood = A.in.hasFood[abl_i];
    abl_out.max_home = A.out.max_home[abl_i];
    abl_out.max_food = A.out.max_food[abl_i];
    ant_deposit(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.reward[abl_i] = abl_out.reward;
    A.out.max_home[abl_i] = abl_out.max_home;
    A.out.max_food[abl_i] = abl_out.max_food;
}
static int abl_launch_ant_deposit(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_ant_deposit A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.pos = (float2 *) L->in_cols[0];
    A.out.pos = (float2 *) L->out_cols[0];
    A.in.last_pos = (float2 *) L->in_cols[1];
    A.out.last_pos = (float2 *) L->out_cols[1];
    A.in.reward = (double *) L->in_cols[2];
    A.out.reward = (double *) L->out_cols[2];
    A.in.max_home = (double *) L->in_cols[3];
    A.out.max_home = (double *) L->out_cols[3];
    A.in.max_food = (double *) L->in_cols[4];
    A.out.max_food = (double *) L->out_cols[4];
    A.in.hasFood = (bool *) L->in_cols[5];
    A.out.hasFood = (bool *) L->out_cols[5];
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
    abl_kernel_ant_deposit<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
__device__ __forceinline__ void abl_ens_body_ant_deposit(const abl_ens_launch &A, long abl_vb, long abl_ts) {
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
            return !(dist_float2(abl_p, abl_p1) > abl_G.pheromone_radius);
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
    Ant abl_in, abl_out;
    abl_in.pos = ((const float2 *) A.in_cols[0])[abl_i];
    abl_in.last_pos = ((const float2 *) A.in_cols[1])[abl_i];
    abl_in.reward = ((const double *) A.in_cols[2])[abl_i];
    abl_in.max_home = ((const double *) A.in_cols[3])[abl_i];
    abl_in.max_food = ((const double *) A.in_cols[4])[abl_i];
    abl_in.hasFood = ((const bool *) A.in_cols[5])[abl_i];
    abl_out.max_home = ((const double *) A.out_cols[3])[abl_i];
    abl_out.max_food = ((const double *) A.out_cols[4])[abl_i];
    ant_deposit(abl_Gr, A.views[abl_r], abl_K, &abl_in, &abl_out);
    ((double *) A.out_cols[2])[abl_i] = abl_out.reward;
    ((double *) A.out_cols[3])[abl_i] = abl_out.max_home;
    ((double *) A.out_cols[4])[abl_i] = abl_out.max_food;
}
#ifndef ABL_PERSIST
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ens_ant_deposit(const __grid_constant__ abl_ens_launch A) {
    abl_ens_body_ant_deposit(A, blockIdx.x, A.timestep);
}
static int abl_launch_ens_ant_deposit(const abl_ens_launch *L, cudaStream_t abl_stream) {
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (L->n + abl_block - 1) / abl_block;
    abl_kernel_ens_ant_deposit<<<abl_grid, abl_block, L->smem, abl_stream>>>(*L);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
#ifndef ABL_PERSIST
static double abl_radius_ant_deposit(const void *abl_gp) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    return (double) (abl_G.pheromone_radius);
}
#endif

__device__ static void pheromone_deposit(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Pheromone* in, Pheromone* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    double food = in->food;
    double home = in->home;
    {
        const abl::near_query<2> abl_q2(abl_NB, (double) in->pos.x, (double) in->pos.y, 0.0, abl_K.self);
        abl::near_list_cursor<2> abl_c2(abl_NB, abl_q2, abl_K);
        auto abl_exact2 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) abl_NB.cols[0])[abl_s];
            return !(dist_float2(abl_p, in->pos) > 0.9);
        };
        while (abl_c2.fill(abl_q2, abl_exact2)) {
            int abl_pslot2 = abl_c2.slot(0);
            Ant abl_pnx2;
            abl_pnx2.max_home = ((const double *) abl_NB.cols[3])[abl_pslot2];
            abl_pnx2.max_food = ((const double *) abl_NB.cols[4])[abl_pslot2];
            abl_pnx2.hasFood = ((const bool *) abl_NB.cols[5])[abl_pslot2];
            for (int abl_k = 0; abl_k < abl_c2.cnt; ++abl_k) {
                const int abl_slot2 = abl_pslot2;
                Ant abl_nx2 = abl_pnx2;
                if (abl_k + 1 < abl_c2.cnt) {
                    abl_pslot2 = abl_c2.slot(abl_k + 1);
                    abl_pnx2.max_home = ((const double *) abl_NB.cols[3])[abl_pslot2];
                    abl_pnx2.max_food = ((const double *) abl_NB.cols[4])[abl_pslot2];
                    abl_pnx2.hasFood = ((const bool *) abl_NB.cols[5])[abl_pslot2];
                }
                Ant* ax = &abl_nx2;
                {
                    if (ax->hasFood) {
                        food = max(ax->max_food, food);
                    } else {
                        home = max(ax->max_home, home);
                    }
                }
            }
        }
    }
    out->food = (food * abl_G.evaporationConstant);
    out->home = (home * abl_G.evaporationConstant);
}

#ifndef ABL_PERSIST
struct abl_kargs_pheromone_deposit {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Pheromone in, out;
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
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_pheromone_deposit(const __grid_constant__ abl_kargs_pheromone_deposit A) {
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
            return !(dist_float2(abl_p, abl_p1) > 0.9);
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
    Pheromone abl_in, abl_out;
    abl_in.pos = A.in.pos[abl_i];
    abl_in.food = A.in.food[abl_i];
    abl_in.home = A.in.home[abl_i];
    pheromone_deposit(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.food[abl_i] = abl_out.food;
    A.out.home[abl_i] = abl_out.home;
}
static int abl_launch_pheromone_deposit(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_pheromone_deposit A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.pos = (float2 *) L->in_cols[0];
    A.out.pos = (float2 *) L->out_cols[0];
    A.in.food = (double *) L->in_cols[1];
    A.out.food = (double *) L->out_cols[1];
    A.in.home = (double *) L->in_cols[2];
    A.out.home = (double *) L->out_cols[2];
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
    abl_kernel_pheromone_deposit<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
__device__ __forceinline__ void abl_ens_body_pheromone_deposit(const abl_ens_launch &A, long abl_vb, long abl_ts) {
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
            return !(dist_float2(abl_p, abl_p1) > 0.9);
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
    Pheromone abl_in, abl_out;
    abl_in.pos = ((const float2 *) A.in_cols[0])[abl_i];
    abl_in.food = ((const double *) A.in_cols[1])[abl_i];
    abl_in.home = ((const double *) A.in_cols[2])[abl_i];
    pheromone_deposit(abl_Gr, A.views[abl_r], abl_K, &abl_in, &abl_out);
    ((double *) A.out_cols[1])[abl_i] = abl_out.food;
    ((double *) A.out_cols[2])[abl_i] = abl_out.home;
}
#ifndef ABL_PERSIST
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ens_pheromone_deposit(const __grid_constant__ abl_ens_launch A) {
    abl_ens_body_pheromone_deposit(A, blockIdx.x, A.timestep);
}
static int abl_launch_ens_pheromone_deposit(const abl_ens_launch *L, cudaStream_t abl_stream) {
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (L->n + abl_block - 1) / abl_block;
    abl_kernel_ens_pheromone_deposit<<<abl_grid, abl_block, L->smem, abl_stream>>>(*L);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
#ifndef ABL_PERSIST
static double abl_radius_pheromone_deposit(const void *abl_gp) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    return (double) (0.9);
}
#endif

__device__ static void ant_act(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Ant* in, Ant* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    float2 new_pos = in->pos;
    double food_max = 0.0;
    double home_max = 0.0;
    float2 food_pos_max = float2_create(0, 0);
    float2 home_pos_max = float2_create(0, 0);
    int same_food_count = 0;
    int same_home_count = 0;
    {
        const abl::near_query<2> abl_q3(abl_NB, (double) in->pos.x, (double) in->pos.y, 0.0, abl_K.self);
        abl::near_list_cursor<2> abl_c3(abl_NB, abl_q3, abl_K);
        auto abl_exact3 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) abl_NB.cols[0])[abl_s];
            return !(dist_float2(abl_p, in->pos) > abl_G.pheromone_radius);
        };
        while (abl_c3.fill(abl_q3, abl_exact3)) {
            int abl_pslot3 = abl_c3.slot(0);
            Pheromone abl_pnx3;
            abl_pnx3.pos = ((const float2 *) abl_NB.cols[0])[abl_pslot3];
            abl_pnx3.food = ((const double *) abl_NB.cols[1])[abl_pslot3];
            abl_pnx3.home = ((const double *) abl_NB.cols[2])[abl_pslot3];
            for (int abl_k = 0; abl_k < abl_c3.cnt; ++abl_k) {
                const int abl_slot3 = abl_pslot3;
                Pheromone abl_nx3 = abl_pnx3;
                if (abl_k + 1 < abl_c3.cnt) {
                    abl_pslot3 = abl_c3.slot(abl_k + 1);
                    abl_pnx3.pos = ((const float2 *) abl_NB.cols[0])[abl_pslot3];
                    abl_pnx3.food = ((const double *) abl_NB.cols[1])[abl_pslot3];
                    abl_pnx3.home = ((const double *) abl_NB.cols[2])[abl_pslot3];
                }
                Pheromone* px = &abl_nx3;
                {
                    if ((px->food > food_max)) {
                        food_max = px->food;
                        food_pos_max = px->pos;
                        same_food_count = 1;
                    } else if (((food_max == px->food) && random_boolean(abl_G, abl_R, (1.0 / (float) (same_food_count + 1))))) {
                        food_max = px->food;
                        food_pos_max = px->pos;
                        same_food_count += 1;
                    }
                    if ((px->home > home_max)) {
                        home_max = px->home;
                        home_pos_max = px->pos;
                        same_home_count = 1;
                    } else if (((home_max == px->home) && random_boolean(abl_G, abl_R, (1.0 / (float) (same_home_count + 1))))) {
                        home_max = px->home;
                        home_pos_max = px->pos;
                        same_home_count += 1;
                    }
                }
            }
        }
    }
    if (in->hasFood) {
        if ((home_max == 0)) new_pos = default_move(abl_G, abl_R, in->pos, in->last_pos); else new_pos = pheromone_move(abl_G, abl_R, in->pos, home_pos_max);
        if (is_home(abl_G, abl_R, new_pos)) {
            out->hasFood = false;
            out->reward = 1.0;
        }
    } else {
        if ((food_max == 0)) new_pos = default_move(abl_G, abl_R, in->pos, in->last_pos); else new_pos = pheromone_move(abl_G, abl_R, in->pos, food_pos_max);
        if (is_food(abl_G, abl_R, new_pos)) {
            out->hasFood = true;
            out->reward = 1.0;
        }
    }
    if ((is_obstacle(abl_G, abl_R, new_pos) || (!is_inside(abl_G, abl_R, new_pos, float2_fill(abl_G.env_size))))) new_pos = in->last_pos;
    out->max_home = home_max;
    out->max_food = food_max;
    out->last_pos = in->pos;
    out->pos = new_pos;
}

#ifndef ABL_PERSIST
struct abl_kargs_ant_act {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Ant in, out;
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
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ant_act(const __grid_constant__ abl_kargs_ant_act A) {
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
            return !(dist_float2(abl_p, abl_p1) > abl_G.pheromone_radius);
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
    Ant abl_in, abl_out;
    abl_in.pos = A.in.pos[abl_i];
    abl_in.last_pos = A.in.last_pos[abl_i];
    abl_in.reward = A.in.reward[abl_i];
    abl_in.max_home = A.in.max_home[abl_i];
    abl_in.max_food = A.in.max_food[abl_i];
    abl_in.hasFood = A.in.hasFood[abl_i];
    abl_out.reward = A.out.reward[abl_i];
    abl_out.hasFood = A.out.hasFood[abl_i];
    ant_act(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.pos[abl_i] = abl_out.pos;
    A.out.last_pos[abl_i] = abl_out.last_pos;
    A.out.reward[abl_i] = abl_out.reward;
    A.out.max_home[abl_i] = abl_out.max_home;
    A.out.max_food[abl_i] = abl_out.max_food;
    A.out.hasFood[abl_i] = abl_out.hasFood;
}
static int abl_launch_ant_act(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_ant_act A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.pos = (float2 *) L->in_cols[0];
    A.out.pos = (float2 *) L->out_cols[0];
    A.in.last_pos = (float2 *) L->in_cols[1];
    A.out.last_pos = (float2 *) L->out_cols[1];
    A.in.reward = (double *) L->in_cols[2];
    A.out.reward = (double *) L->out_cols[2];
    A.in.max_home = (double *) L->in_cols[3];
    A.out.max_home = (double *) L->out_cols[3];
    A.in.max_food = (double *) L->in_cols[4];
    A.out.max_food = (double *) L->out_cols[4];
    A.in.hasFood = (bool *) L->in_cols[5];
    A.out.hasFood = (bool *) L->out_cols[5];
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
    abl_kernel_ant_act<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
__device__ __forceinline__ void abl_ens_body_ant_act(const abl_ens_launch &A, long abl_vb, long abl_ts) {
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
            return !(dist_float2(abl_p, abl_p1) > abl_G.pheromone_radius);
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
    Ant abl_in, abl_out;
    abl_in.pos = ((const float2 *) A.in_cols[0])[abl_i];
    abl_in.last_pos = ((const float2 *) A.in_cols[1])[abl_i];
    abl_in.reward = ((const double *) A.in_cols[2])[abl_i];
    abl_in.max_home = ((const double *) A.in_cols[3])[abl_i];
    abl_in.max_food = ((const double *) A.in_cols[4])[abl_i];
    abl_in.hasFood = ((const bool *) A.in_cols[5])[abl_i];
    abl_out.reward = ((const double *) A.out_cols[2])[abl_i];
    abl_out.hasFood = ((const bool *) A.out_cols[5])[abl_i];
    ant_act(abl_Gr, A.views[abl_r], abl_K, &abl_in, &abl_out);
    ((float2 *) A.out_cols[0])[abl_i] = abl_out.pos;
    ((float2 *) A.out_cols[1])[abl_i] = abl_out.last_pos;
    ((double *) A.out_cols[2])[abl_i] = abl_out.reward;
    ((double *) A.out_cols[3])[abl_i] = abl_out.max_home;
    ((double *) A.out_cols[4])[abl_i] = abl_out.max_food;
    ((bool *) A.out_cols[5])[abl_i] = abl_out.hasFood;
}
#ifndef ABL_PERSIST
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ens_ant_act(const __grid_constant__ abl_ens_launch A) {
    abl_ens_body_ant_act(A, blockIdx.x, A.timestep);
}
static int abl_launch_ens_ant_act(const abl_ens_launch *L, cudaStream_t abl_stream) {
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (L->n + abl_block - 1) / abl_block;
    abl_kernel_ens_ant_act<<<abl_grid, abl_block, L->smem, abl_stream>>>(*L);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
#ifndef ABL_PERSIST
static double abl_radius_ant_act(const void *abl_gp) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    return (double) (abl_G.pheromone_radius);
}
#endif


#ifndef ABL_PERSIST
extern "C" int abl_persist_launch_ants(const void *, int *, int, size_t, int *, cudaStream_t);
static const abl_member_desc abl_members_Ant[] = {
    {"pos", ABL_T_FLOAT2, 2, 8, 1},
    {"last_pos", ABL_T_FLOAT2, 2, 8, 0},
    {"reward", ABL_T_FLOAT, 1, 8, 0},
    {"max_home", ABL_T_FLOAT, 1, 8, 0},
    {"max_food", ABL_T_FLOAT, 1, 8, 0},
    {"hasFood", ABL_T_BOOL, 1, 1, 0},
};
static const abl_member_desc abl_members_Pheromone[] = {
    {"pos", ABL_T_FLOAT2, 2, 8, 1},
    {"food", ABL_T_FLOAT, 1, 8, 0},
    {"home", ABL_T_FLOAT, 1, 8, 0},
};
static const abl_agent_desc abl_agents[] = {
    {"Ant", 6, abl_members_Ant, 0, 2},
    {"Pheromone", 3, abl_members_Pheromone, 0, 2},
};
static const abl_global_desc abl_global_table[] = {
    {"PI", ABL_T_FLOAT, offsetof(abl_globals, PI)},
    {"SQRT2", ABL_T_FLOAT, offsetof(abl_globals, SQRT2)},
    {"evaporationConstant", ABL_T_FLOAT, offsetof(abl_globals, evaporationConstant)},
    {"initialReward", ABL_T_FLOAT, offsetof(abl_globals, initialReward)},
    {"cutDown", ABL_T_FLOAT, offsetof(abl_globals, cutDown)},
    {"momentumProbability", ABL_T_FLOAT, offsetof(abl_globals, momentumProbability)},
    {"randomActionProbability", ABL_T_FLOAT, offsetof(abl_globals, randomActionProbability)},
    {"pheromone_radius", ABL_T_FLOAT, offsetof(abl_globals, pheromone_radius)},
    {"ants_density", ABL_T_FLOAT, offsetof(abl_globals, ants_density)},
    {"num_agents", ABL_T_INT, offsetof(abl_globals, num_agents)},
    {"num_timesteps", ABL_T_INT, offsetof(abl_globals, num_timesteps)},
    {"num_ants", ABL_T_INT, offsetof(abl_globals, num_ants)},
    {"env_size", ABL_T_INT, offsetof(abl_globals, env_size)},
    {"num_pheromones", ABL_T_INT, offsetof(abl_globals, num_pheromones)},
    {"env_scale", ABL_T_FLOAT, offsetof(abl_globals, env_scale)},
    {"home_pos", ABL_T_FLOAT2, offsetof(abl_globals, home_pos)},
    {"food_pos", ABL_T_FLOAT2, offsetof(abl_globals, food_pos)},
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
    {"ant_deposit", 0, 1, 1, abl_radius_ant_deposit, 7u, 4u, abl_launch_ant_deposit, 0, -1, 0, abl_launch_ens_ant_deposit, 0, 1, 28u, 1},
    {"pheromone_deposit", 1, 0, 1, abl_radius_pheromone_deposit, 57u, 6u, abl_launch_pheromone_deposit, 0, -1, 0, abl_launch_ens_pheromone_deposit, 0, 1, 6u, 1},
    {"ant_act", 0, 1, 1, abl_radius_ant_act, 7u, 27u, abl_launch_ant_act, 0, -1, 0, abl_launch_ens_ant_act, 1, 1, 63u, 1},
};
static const abl_step_desc abl_steps_ordered[] = {
    abl_steps[0],
    abl_steps[1],
    abl_steps[2],
    {nullptr, 0, -1, 0, nullptr, 0u, 0u, nullptr, 0, -1, 0, nullptr, 0}
};
extern const abl_model_desc abl_desc = {
    "ants", 2, abl_agents, 3, abl_steps_ordered, sizeof(abl_globals), &abl_globals_default, 17, abl_global_table, 2, abl_env_bounds, nullptr, 0, nullptr, abl_persist_launch_ants
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
        size_t n = agents.agents_Ant.len;
        const Ant *aos = (const Ant *) agents.agents_Ant.values;
        float2 *c0 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c0[i] = aos[i].pos;
        float2 *c1 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c1[i] = aos[i].last_pos;
        double *c2 = (double *) std::malloc(sizeof(double) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c2[i] = aos[i].reward;
        double *c3 = (double *) std::malloc(sizeof(double) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c3[i] = aos[i].max_home;
        double *c4 = (double *) std::malloc(sizeof(double) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c4[i] = aos[i].max_food;
        bool *c5 = (bool *) std::malloc(sizeof(bool) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c5[i] = aos[i].hasFood;
        const void *cols[] = {c0, c1, c2, c3, c4, c5};
        abl_check(abl_upload(ctx, 0, cols, n), "abl_upload");
        std::free(c0);
        std::free(c1);
        std::free(c2);
        std::free(c3);
        std::free(c4);
        std::free(c5);
    }
    {
        size_t n = agents.agents_Pheromone.len;
        const Pheromone *aos = (const Pheromone *) agents.agents_Pheromone.values;
        float2 *c0 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c0[i] = aos[i].pos;
        double *c1 = (double *) std::malloc(sizeof(double) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c1[i] = aos[i].food;
        double *c2 = (double *) std::malloc(sizeof(double) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c2[i] = aos[i].home;
        const void *cols[] = {c0, c1, c2};
        abl_check(abl_upload(ctx, 1, cols, n), "abl_upload");
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
        double *c2 = (double *) std::malloc(sizeof(double) * (n ? n : 1));
        double *c3 = (double *) std::malloc(sizeof(double) * (n ? n : 1));
        double *c4 = (double *) std::malloc(sizeof(double) * (n ? n : 1));
        bool *c5 = (bool *) std::malloc(sizeof(bool) * (n ? n : 1));
        void *cols[] = {c0, c1, c2, c3, c4, c5};
        size_t cap = n;
        abl_check(abl_download(ctx, 0, cols, &cap), "abl_download");
        dyn_array_clean(&agents.agents_Ant);
        agents.agents_Ant = dyn_array_create_fixed(sizeof(Ant), n);
        Ant *aos = (Ant *) agents.agents_Ant.values;
        for (size_t i = 0; i < n; i++) {
            aos[i].pos = c0[i];
            aos[i].last_pos = c1[i];
            aos[i].reward = c2[i];
            aos[i].max_home = c3[i];
            aos[i].max_food = c4[i];
            aos[i].hasFood = c5[i];
        }
        std::free(c0);
        std::free(c1);
        std::free(c2);
        std::free(c3);
        std::free(c4);
        std::free(c5);
    }
    {
        size_t n = 0;
        abl_check(abl_count(ctx, 1, &n), "abl_count");
        float2 *c0 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        double *c1 = (double *) std::malloc(sizeof(double) * (n ? n : 1));
        double *c2 = (double *) std::malloc(sizeof(double) * (n ? n : 1));
        void *cols[] = {c0, c1, c2};
        size_t cap = n;
        abl_check(abl_download(ctx, 1, cols, &cap), "abl_download");
        dyn_array_clean(&agents.agents_Pheromone);
        agents.agents_Pheromone = dyn_array_create_fixed(sizeof(Pheromone), n);
        Pheromone *aos = (Pheromone *) agents.agents_Pheromone.values;
        for (size_t i = 0; i < n; i++) {
            aos[i].pos = c0[i];
            aos[i].food = c1[i];
            aos[i].home = c2[i];
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
    for (int i = 0, _var0 = abl_G.env_size; i < _var0; ++i) {
        for (int j = 0, _var1 = abl_G.env_size; j < _var1; ++j) {
            *DYN_ARRAY_PLACE(&agents.agents_Pheromone, Pheromone) = ([&]() { Pheromone abl_a; abl_a.pos = float2_create(((float) i + 0.5), ((float) j + 0.5)); abl_a.food = 0.0; abl_a.home = 0.0; return abl_a; }());
        }
    }
    for (int i = 0, _var2 = abl_G.num_ants; i < _var2; ++i) {
        float2 pos = abl_G.home_pos;
        *DYN_ARRAY_PLACE(&agents.agents_Ant, Ant) = ([&]() { Ant abl_a; abl_a.pos = pos; abl_a.last_pos = pos; abl_a.reward = abl_G.initialReward; abl_a.max_home = 0.0; abl_a.max_food = 0.0; abl_a.hasFood = false; return abl_a; }());
    }
    abl_simulate(abl_G.num_timesteps);
    save(&agents, agents_info, "ants.out", SAVE_JSON);
    return 0;
}
#else
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_PERSIST_MIN_BLOCKS) abl_kernel_ens_persist(const abl::persist_prog *abl_P, int *abl_err) {
    abl::persist_run<abl_float, 2>(abl_P, abl_err, [&](const abl_ens_launch &abl_L, long abl_vb, long abl_ts) {
        switch (abl_L.step_index) {
            case 0: abl_ens_body_ant_deposit(abl_L, abl_vb, abl_ts); break;
            case 1: abl_ens_body_pheromone_deposit(abl_L, abl_vb, abl_ts); break;
            case 2: abl_ens_body_ant_act(abl_L, abl_vb, abl_ts); break;
            default: break;
        }
    });
}
#endif

}  // namespace abl_model_ants

#ifdef ABL_PERSIST
extern "C" int abl_persist_launch_ants(const void *abl_prog, int *abl_err, int abl_block, size_t abl_smem, int *abl_grid, cudaStream_t abl_stream) {
    return abl::persist_launch((const void *) abl_model_ants::abl_kernel_ens_persist, abl_prog, abl_err, abl_block, abl_smem, abl_grid, abl_stream);
}
#endif
#ifndef ABL_PERSIST
extern "C" const abl_model_desc *abl_model_desc_ants(void) {
    return &abl_model_ants::abl_desc;
}
#endif

#if defined(ABL_STANDALONE_MAIN) && !defined(ABL_PERSIST)
extern "C" const abl_model_desc *const abl_builtin_models[] = {
    &abl_model_ants::abl_desc, nullptr};
int main() { return abl_model_ants::abl_main(); }
#endif
