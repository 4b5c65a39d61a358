// Generated by OpenABL -b cuda (model "sugarscape").
#include "abl_gen.cuh"

namespace abl_model_sugarscape {

typedef double abl_float;
#include "abl_math.cuh"

typedef struct {
    float2 pos;
    float2 target_pos;
    int agent_id;
    int state;
    int sugar_level;
    int metabolism;
    int env_sugar_level;
    int max_env_sugar_level;
} Agent;
static const type_info Agent_info[] = {
    { TYPE_FLOAT2, offsetof(Agent, pos), "pos", true },
    { TYPE_FLOAT2, offsetof(Agent, target_pos), "target_pos", false },
    { TYPE_INT, offsetof(Agent, agent_id), "agent_id", false },
    { TYPE_INT, offsetof(Agent, state), "state", false },
    { TYPE_INT, offsetof(Agent, sugar_level), "sugar_level", false },
    { TYPE_INT, offsetof(Agent, metabolism), "metabolism", false },
    { TYPE_INT, offsetof(Agent, env_sugar_level), "env_sugar_level", false },
    { TYPE_INT, offsetof(Agent, max_env_sugar_level), "max_env_sugar_level", false },
    { TYPE_END, sizeof(Agent), NULL }
};

struct agent_struct {
    dyn_array agents_Agent;
    dyn_array agents_Agent_dbuf;
};
static struct agent_struct agents;
static const agent_info agents_info[] = {
    { Agent_info, offsetof(struct agent_struct, agents_Agent), "Agent" },
    { NULL, 0, NULL }
};

struct abl_globals {
    double PI;
    int AGENT_STATE_UNOCCUPIED;
    int AGENT_STATE_OCCUPIED;
    int AGENT_STATE_MOVEMENT_REQUESTED;
    int AGENT_STATE_MOVEMENT_UNRESOLVED;
    int SUGAR_GROWBACK_RATE;
    int min_start_sugar_level;
    int max_start_sugar_level;
    double radius;
    int num_timesteps;
    double occupiedFrac;
    int num_agents;
    int grid_width;
    float2 sugar_center1;
    float2 sugar_center2;
    int global_max_env_sugar_level;
    double sugar_variance;
};
static const abl_globals abl_globals_default = {
    3.14159,
    0,
    1,
    2,
    3,
    1,
    1,
    10,
    1.5,
    100,
    0.1,
    10000,
    100,
    {25.0, 25.0},
    {75.0, 75.0},
    50,
    250.0,
};
static abl_globals abl_G = abl_globals_default;
static abl::rng abl_R;  // unused on the host: main() draws from the host stream
struct abl_cols_Agent {
    float2 *pos;
    float2 *target_pos;
    int *agent_id;
    int *state;
    int *sugar_level;
    int *metabolism;
    int *env_sugar_level;
    int *max_env_sugar_level;
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
__device__ static void metabolise_and_growback(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Agent* in, Agent* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    int new_env_sugar_level = in->env_sugar_level;
    if ((in->state == abl_G.AGENT_STATE_OCCUPIED)) {
        int new_sugar_level = ((in->sugar_level + in->env_sugar_level) - in->metabolism);
        new_env_sugar_level = 0;
        if ((new_sugar_level <= 0)) {
            out->state = abl_G.AGENT_STATE_UNOCCUPIED;
            out->agent_id = (-1);
            out->sugar_level = 0;
            out->metabolism = 0;
        } else {
            out->state = abl_G.AGENT_STATE_MOVEMENT_UNRESOLVED;
            out->sugar_level = new_sugar_level;
        }
    }
    new_env_sugar_level += abl_G.SUGAR_GROWBACK_RATE;
    if ((new_env_sugar_level > in->max_env_sugar_level)) {
        new_env_sugar_level = in->max_env_sugar_level;
    }
    out->env_sugar_level = new_env_sugar_level;
}

#ifndef ABL_PERSIST
struct abl_kargs_metabolise_and_growback {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Agent in, out;
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
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_metabolise_and_growback(const __grid_constant__ abl_kargs_metabolise_and_growback A) {
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
    Agent abl_in, abl_out;
    abl_in.pos = A.in.pos[abl_i];
    abl_in.target_pos = A.in.target_pos[abl_i];
    abl_in.agent_id = A.in.agent_id[abl_i];
    abl_in.state = A.in.state[abl_i];
    abl_in.sugar_level = A.in.sugar_level[abl_i];
    abl_in.metabolism = A.in.metabolism[abl_i];
    abl_in.env_sugar_level = A.in.env_sugar_level[abl_i];
    abl_in.max_env_sugar_level = A.in.max_env_sugar_level[abl_i];
    abl_out.agent_id = A.out.agent_id[abl_i];
    abl_out.state = A.out.state[abl_i];
    abl_out.sugar_level = A.out.sugar_level[abl_i];
    abl_out.metabolism = A.out.metabolism[abl_i];
    metabolise_and_growback(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.agent_id[abl_i] = abl_out.agent_id;
    A.out.state[abl_i] = abl_out.state;
    A.out.sugar_level[abl_i] = abl_out.sugar_level;
    A.out.metabolism[abl_i] = abl_out.metabolism;
    A.out.env_sugar_level[abl_i] = abl_out.env_sugar_level;
}
static int abl_launch_metabolise_and_growback(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_metabolise_and_growback A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.pos = (float2 *) L->in_cols[0];
    A.out.pos = (float2 *) L->out_cols[0];
    A.in.target_pos = (float2 *) L->in_cols[1];
    A.out.target_pos = (float2 *) L->out_cols[1];
    A.in.agent_id = (int *) L->in_cols[2];
    A.out.agent_id = (int *) L->out_cols[2];
    A.in.state = (int *) L->in_cols[3];
    A.out.state = (int *) L->out_cols[3];
    A.in.sugar_level = (int *) L->in_cols[4];
    A.out.sugar_level = (int *) L->out_cols[4];
    A.in.metabolism = (int *) L->in_cols[5];
    A.out.metabolism = (int *) L->out_cols[5];
    A.in.env_sugar_level = (int *) L->in_cols[6];
    A.out.env_sugar_level = (int *) L->out_cols[6];
    A.in.max_env_sugar_level = (int *) L->in_cols[7];
    A.out.max_env_sugar_level = (int *) L->out_cols[7];
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
    abl_kernel_metabolise_and_growback<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
__device__ __forceinline__ void abl_ens_body_metabolise_and_growback(const abl_ens_launch &A, long abl_vb, long abl_ts) {
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
    Agent abl_in, abl_out;
    abl_in.pos = ((const float2 *) A.in_cols[0])[abl_i];
    abl_in.target_pos = ((const float2 *) A.in_cols[1])[abl_i];
    abl_in.agent_id = ((const int *) A.in_cols[2])[abl_i];
    abl_in.state = ((const int *) A.in_cols[3])[abl_i];
    abl_in.sugar_level = ((const int *) A.in_cols[4])[abl_i];
    abl_in.metabolism = ((const int *) A.in_cols[5])[abl_i];
    abl_in.env_sugar_level = ((const int *) A.in_cols[6])[abl_i];
    abl_in.max_env_sugar_level = ((const int *) A.in_cols[7])[abl_i];
    abl_out.agent_id = ((const int *) A.out_cols[2])[abl_i];
    abl_out.state = ((const int *) A.out_cols[3])[abl_i];
    abl_out.sugar_level = ((const int *) A.out_cols[4])[abl_i];
    abl_out.metabolism = ((const int *) A.out_cols[5])[abl_i];
    metabolise_and_growback(abl_Gr, A.views[abl_r], abl_K, &abl_in, &abl_out);
    ((int *) A.out_cols[2])[abl_i] = abl_out.agent_id;
    ((int *) A.out_cols[3])[abl_i] = abl_out.state;
    ((int *) A.out_cols[4])[abl_i] = abl_out.sugar_level;
    ((int *) A.out_cols[5])[abl_i] = abl_out.metabolism;
    ((int *) A.out_cols[6])[abl_i] = abl_out.env_sugar_level;
}
#ifndef ABL_PERSIST
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ens_metabolise_and_growback(const __grid_constant__ abl_ens_launch A) {
    abl_ens_body_metabolise_and_growback(A, blockIdx.x, A.timestep);
}
static int abl_launch_ens_metabolise_and_growback(const abl_ens_launch *L, cudaStream_t abl_stream) {
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (L->n + abl_block - 1) / abl_block;
    abl_kernel_ens_metabolise_and_growback<<<abl_grid, abl_block, L->smem, abl_stream>>>(*L);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif

__device__ static void movement_request(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Agent* in, Agent* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    if ((in->state == abl_G.AGENT_STATE_MOVEMENT_UNRESOLVED)) {
        int best_sugar_level = (-1);
        float2 best_pos = float2_fill(0);
        {
            const abl::near_query<2> abl_q1(abl_NB, (double) in->pos.x, (double) in->pos.y, 0.0, abl_K.self);
            abl::near_list_cursor<2> abl_c1(abl_NB, abl_q1, abl_K);
            auto abl_exact1 = [&](int abl_s) -> bool {
                const float2 abl_p = ((const float2 *) abl_NB.cols[0])[abl_s];
                return !(dist_float2(abl_p, in->pos) > abl_G.radius);
            };
            while (abl_c1.fill(abl_q1, abl_exact1)) {
                int abl_pslot1 = abl_c1.slot(0);
                Agent abl_pnx1;
                abl_pnx1.pos = ((const float2 *) abl_NB.cols[0])[abl_pslot1];
                abl_pnx1.state = ((const int *) abl_NB.cols[3])[abl_pslot1];
                abl_pnx1.env_sugar_level = ((const int *) abl_NB.cols[6])[abl_pslot1];
                for (int abl_k = 0; abl_k < abl_c1.cnt; ++abl_k) {
                    const int abl_slot1 = abl_pslot1;
                    Agent abl_nx1 = abl_pnx1;
                    if (abl_k + 1 < abl_c1.cnt) {
                        abl_pslot1 = abl_c1.slot(abl_k + 1);
                        abl_pnx1.pos = ((const float2 *) abl_NB.cols[0])[abl_pslot1];
                        abl_pnx1.state = ((const int *) abl_NB.cols[3])[abl_pslot1];
                        abl_pnx1.env_sugar_level = ((const int *) abl_NB.cols[6])[abl_pslot1];
                    }
                    Agent* nx = &abl_nx1;
                    {
                        if (float2_equals(nx->pos, in->pos)) continue;
                        if (((nx->state == abl_G.AGENT_STATE_UNOCCUPIED) && (nx->env_sugar_level > best_sugar_level))) {
                            best_sugar_level = nx->env_sugar_level;
                            best_pos = nx->pos;
                        }
                    }
                }
            }
        }
        if ((best_sugar_level > in->env_sugar_level)) {
            out->state = abl_G.AGENT_STATE_MOVEMENT_REQUESTED;
            out->target_pos = best_pos;
        } else {
            out->state = abl_G.AGENT_STATE_OCCUPIED;
        }
    }
}

#ifndef ABL_PERSIST
struct abl_kargs_movement_request {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Agent in, out;
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
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_movement_request(const __grid_constant__ abl_kargs_movement_request A) {
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
            return !(dist_float2(abl_p, abl_p1) > abl_G.radius);
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
    Agent abl_in, abl_out;
    abl_in.pos = A.in.pos[abl_i];
    abl_in.target_pos = A.in.target_pos[abl_i];
    abl_in.agent_id = A.in.agent_id[abl_i];
    abl_in.state = A.in.state[abl_i];
    abl_in.sugar_level = A.in.sugar_level[abl_i];
    abl_in.metabolism = A.in.metabolism[abl_i];
    abl_in.env_sugar_level = A.in.env_sugar_level[abl_i];
    abl_in.max_env_sugar_level = A.in.max_env_sugar_level[abl_i];
    abl_out.target_pos = A.out.target_pos[abl_i];
    abl_out.state = A.out.state[abl_i];
    movement_request(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.target_pos[abl_i] = abl_out.target_pos;
    A.out.state[abl_i] = abl_out.state;
}
static int abl_launch_movement_request(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_movement_request A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.pos = (float2 *) L->in_cols[0];
    A.out.pos = (float2 *) L->out_cols[0];
    A.in.target_pos = (float2 *) L->in_cols[1];
    A.out.target_pos = (float2 *) L->out_cols[1];
    A.in.agent_id = (int *) L->in_cols[2];
    A.out.agent_id = (int *) L->out_cols[2];
    A.in.state = (int *) L->in_cols[3];
    A.out.state = (int *) L->out_cols[3];
    A.in.sugar_level = (int *) L->in_cols[4];
    A.out.sugar_level = (int *) L->out_cols[4];
    A.in.metabolism = (int *) L->in_cols[5];
    A.out.metabolism = (int *) L->out_cols[5];
    A.in.env_sugar_level = (int *) L->in_cols[6];
    A.out.env_sugar_level = (int *) L->out_cols[6];
    A.in.max_env_sugar_level = (int *) L->in_cols[7];
    A.out.max_env_sugar_level = (int *) L->out_cols[7];
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
    abl_kernel_movement_request<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
__device__ __forceinline__ void abl_ens_body_movement_request(const abl_ens_launch &A, long abl_vb, long abl_ts) {
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
            return !(dist_float2(abl_p, abl_p1) > abl_G.radius);
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
    Agent abl_in, abl_out;
    abl_in.pos = ((const float2 *) A.in_cols[0])[abl_i];
    abl_in.target_pos = ((const float2 *) A.in_cols[1])[abl_i];
    abl_in.agent_id = ((const int *) A.in_cols[2])[abl_i];
    abl_in.state = ((const int *) A.in_cols[3])[abl_i];
    abl_in.sugar_level = ((const int *) A.in_cols[4])[abl_i];
    abl_in.metabolism = ((const int *) A.in_cols[5])[abl_i];
    abl_in.env_sugar_level = ((const int *) A.in_cols[6])[abl_i];
    abl_in.max_env_sugar_level = ((const int *) A.in_cols[7])[abl_i];
    abl_out.target_pos = ((const float2 *) A.out_cols[1])[abl_i];
    abl_out.state = ((const int *) A.out_cols[3])[abl_i];
    movement_request(abl_Gr, A.views[abl_r], abl_K, &abl_in, &abl_out);
    ((float2 *) A.out_cols[1])[abl_i] = abl_out.target_pos;
    ((int *) A.out_cols[3])[abl_i] = abl_out.state;
}
#ifndef ABL_PERSIST
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ens_movement_request(const __grid_constant__ abl_ens_launch A) {
    abl_ens_body_movement_request(A, blockIdx.x, A.timestep);
}
static int abl_launch_ens_movement_request(const abl_ens_launch *L, cudaStream_t abl_stream) {
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (L->n + abl_block - 1) / abl_block;
    abl_kernel_ens_movement_request<<<abl_grid, abl_block, L->smem, abl_stream>>>(*L);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
#ifndef ABL_PERSIST
static double abl_radius_movement_request(const void *abl_gp) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    return (double) (abl_G.radius);
}
#endif

__device__ static void movement_response(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Agent* in, Agent* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    if ((in->state == abl_G.AGENT_STATE_UNOCCUPIED)) {
        int best_priority = (-1);
        int best_agent_id = (-1);
        int best_sugar_level = (-1);
        int best_metabolism = (-1);
        {
            const abl::near_query<2> abl_q2(abl_NB, (double) in->pos.x, (double) in->pos.y, 0.0, abl_K.self);
            abl::near_list_cursor<2> abl_c2(abl_NB, abl_q2, abl_K);
            auto abl_exact2 = [&](int abl_s) -> bool {
                const float2 abl_p = ((const float2 *) abl_NB.cols[0])[abl_s];
                return !(dist_float2(abl_p, in->pos) > abl_G.radius);
            };
            while (abl_c2.fill(abl_q2, abl_exact2)) {
                int abl_pslot2 = abl_c2.slot(0);
                Agent abl_pnx2;
                abl_pnx2.target_pos = ((const float2 *) abl_NB.cols[1])[abl_pslot2];
                abl_pnx2.agent_id = ((const int *) abl_NB.cols[2])[abl_pslot2];
                abl_pnx2.state = ((const int *) abl_NB.cols[3])[abl_pslot2];
                abl_pnx2.sugar_level = ((const int *) abl_NB.cols[4])[abl_pslot2];
                abl_pnx2.metabolism = ((const int *) abl_NB.cols[5])[abl_pslot2];
                for (int abl_k = 0; abl_k < abl_c2.cnt; ++abl_k) {
                    const int abl_slot2 = abl_pslot2;
                    Agent abl_nx2 = abl_pnx2;
                    if (abl_k + 1 < abl_c2.cnt) {
                        abl_pslot2 = abl_c2.slot(abl_k + 1);
                        abl_pnx2.target_pos = ((const float2 *) abl_NB.cols[1])[abl_pslot2];
                        abl_pnx2.agent_id = ((const int *) abl_NB.cols[2])[abl_pslot2];
                        abl_pnx2.state = ((const int *) abl_NB.cols[3])[abl_pslot2];
                        abl_pnx2.sugar_level = ((const int *) abl_NB.cols[4])[abl_pslot2];
                        abl_pnx2.metabolism = ((const int *) abl_NB.cols[5])[abl_pslot2];
                    }
                    Agent* nx = &abl_nx2;
                    {
                        if (((nx->state == abl_G.AGENT_STATE_MOVEMENT_REQUESTED) && float2_equals(nx->target_pos, in->pos))) {
                            int message_priority = 0;
                            if ((message_priority > best_priority)) {
                                best_priority = message_priority;
                                best_agent_id = nx->agent_id;
                                best_sugar_level = nx->sugar_level;
                                best_metabolism = nx->metabolism;
                            }
                        }
                    }
                }
            }
        }
        if ((best_agent_id >= 0)) {
            out->state = abl_G.AGENT_STATE_OCCUPIED;
            out->agent_id = best_agent_id;
            out->sugar_level = best_sugar_level;
            out->metabolism = best_metabolism;
        }
    }
}

#ifndef ABL_PERSIST
struct abl_kargs_movement_response {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Agent in, out;
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
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_movement_response(const __grid_constant__ abl_kargs_movement_response A) {
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
            return !(dist_float2(abl_p, abl_p1) > abl_G.radius);
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
    Agent abl_in, abl_out;
    abl_in.pos = A.in.pos[abl_i];
    abl_in.target_pos = A.in.target_pos[abl_i];
    abl_in.agent_id = A.in.agent_id[abl_i];
    abl_in.state = A.in.state[abl_i];
    abl_in.sugar_level = A.in.sugar_level[abl_i];
    abl_in.metabolism = A.in.metabolism[abl_i];
    abl_in.env_sugar_level = A.in.env_sugar_level[abl_i];
    abl_in.max_env_sugar_level = A.in.max_env_sugar_level[abl_i];
    abl_out.agent_id = A.out.agent_id[abl_i];
    abl_out.state = A.out.state[abl_i];
    abl_out.sugar_level = A.out.sugar_level[abl_i];
    abl_out.metabolism = A.out.metabolism[abl_i];
    movement_response(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.agent_id[abl_i] = abl_out.agent_id;
    A.out.state[abl_i] = abl_out.state;
    A.out.sugar_level[abl_i] = abl_out.sugar_level;
    A.out.metabolism[abl_i] = abl_out.metabolism;
}
static int abl_launch_movement_response(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_movement_response A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.pos = (float2 *) L->in_cols[0];
    A.out.pos = (float2 *) L->out_cols[0];
    A.in.target_pos = (float2 *) L->in_cols[1];
    A.out.target_pos = (float2 *) L->out_cols[1];
    A.in.agent_id = (int *) L->in_cols[2];
    A.out.agent_id = (int *) L->out_cols[2];
    A.in.state = (int *) L->in_cols[3];
    A.out.state = (int *) L->out_cols[3];
    A.in.sugar_level = (int *) L->in_cols[4];
    A.out.sugar_level = (int *) L->out_cols[4];
    A.in.metabolism = (int *) L->in_cols[5];
    A.out.metabolism = (int *) L->out_cols[5];
    A.in.env_sugar_level = (int *) L->in_cols[6];
    A.out.env_sugar_level = (int *) L->out_cols[6];
    A.in.max_env_sugar_level = (int *) L->in_cols[7];
    A.out.max_env_sugar_level = (int *) L->out_cols[7];
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
    abl_kernel_movement_response<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
__device__ __forceinline__ void abl_ens_body_movement_response(const abl_ens_launch &A, long abl_vb, long abl_ts) {
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
            return !(dist_float2(abl_p, abl_p1) > abl_G.radius);
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
    Agent abl_in, abl_out;
    abl_in.pos = ((const float2 *) A.in_cols[0])[abl_i];
    abl_in.target_pos = ((const float2 *) A.in_cols[1])[abl_i];
    abl_in.agent_id = ((const int *) A.in_cols[2])[abl_i];
    abl_in.state = ((const int *) A.in_cols[3])[abl_i];
    abl_in.sugar_level = ((const int *) A.in_cols[4])[abl_i];
    abl_in.metabolism = ((const int *) A.in_cols[5])[abl_i];
    abl_in.env_sugar_level = ((const int *) A.in_cols[6])[abl_i];
    abl_in.max_env_sugar_level = ((const int *) A.in_cols[7])[abl_i];
    abl_out.agent_id = ((const int *) A.out_cols[2])[abl_i];
    abl_out.state = ((const int *) A.out_cols[3])[abl_i];
    abl_out.sugar_level = ((const int *) A.out_cols[4])[abl_i];
    abl_out.metabolism = ((const int *) A.out_cols[5])[abl_i];
    movement_response(abl_Gr, A.views[abl_r], abl_K, &abl_in, &abl_out);
    ((int *) A.out_cols[2])[abl_i] = abl_out.agent_id;
    ((int *) A.out_cols[3])[abl_i] = abl_out.state;
    ((int *) A.out_cols[4])[abl_i] = abl_out.sugar_level;
    ((int *) A.out_cols[5])[abl_i] = abl_out.metabolism;
}
#ifndef ABL_PERSIST
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ens_movement_response(const __grid_constant__ abl_ens_launch A) {
    abl_ens_body_movement_response(A, blockIdx.x, A.timestep);
}
static int abl_launch_ens_movement_response(const abl_ens_launch *L, cudaStream_t abl_stream) {
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (L->n + abl_block - 1) / abl_block;
    abl_kernel_ens_movement_response<<<abl_grid, abl_block, L->smem, abl_stream>>>(*L);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
#ifndef ABL_PERSIST
static double abl_radius_movement_response(const void *abl_gp) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    return (double) (abl_G.radius);
}
#endif

__device__ static void movement_transaction(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Agent* in, Agent* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    if ((in->state == abl_G.AGENT_STATE_MOVEMENT_REQUESTED)) {
        bool moved = false;
        {
            const abl::near_query<2> abl_q3(abl_NB, (double) in->pos.x, (double) in->pos.y, 0.0, abl_K.self);
            abl::near_list_cursor<2> abl_c3(abl_NB, abl_q3, abl_K);
            auto abl_exact3 = [&](int abl_s) -> bool {
                const float2 abl_p = ((const float2 *) abl_NB.cols[0])[abl_s];
                return !(dist_float2(abl_p, in->pos) > abl_G.radius);
            };
            while (abl_c3.fill(abl_q3, abl_exact3)) {
                int abl_pslot3 = abl_c3.slot(0);
                Agent abl_pnx3;
                abl_pnx3.agent_id = ((const int *) abl_NB.cols[2])[abl_pslot3];
                abl_pnx3.state = ((const int *) abl_NB.cols[3])[abl_pslot3];
                for (int abl_k = 0; abl_k < abl_c3.cnt; ++abl_k) {
                    const int abl_slot3 = abl_pslot3;
                    Agent abl_nx3 = abl_pnx3;
                    if (abl_k + 1 < abl_c3.cnt) {
                        abl_pslot3 = abl_c3.slot(abl_k + 1);
                        abl_pnx3.agent_id = ((const int *) abl_NB.cols[2])[abl_pslot3];
                        abl_pnx3.state = ((const int *) abl_NB.cols[3])[abl_pslot3];
                    }
                    Agent* nx = &abl_nx3;
                    {
                        if (((nx->state == abl_G.AGENT_STATE_OCCUPIED) && (nx->agent_id == in->agent_id))) {
                            moved = true;
                            out->state = abl_G.AGENT_STATE_UNOCCUPIED;
                            out->agent_id = (-1);
                            out->sugar_level = 0;
                            out->metabolism = 0;
                        }
                    }
                }
            }
        }
        if ((!moved)) {
            out->state = abl_G.AGENT_STATE_OCCUPIED;
        }
    }
}

#ifndef ABL_PERSIST
struct abl_kargs_movement_transaction {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Agent in, out;
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
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_movement_transaction(const __grid_constant__ abl_kargs_movement_transaction A) {
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
            return !(dist_float2(abl_p, abl_p1) > abl_G.radius);
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
    Agent abl_in, abl_out;
    abl_in.pos = A.in.pos[abl_i];
    abl_in.target_pos = A.in.target_pos[abl_i];
    abl_in.agent_id = A.in.agent_id[abl_i];
    abl_in.state = A.in.state[abl_i];
    abl_in.sugar_level = A.in.sugar_level[abl_i];
    abl_in.metabolism = A.in.metabolism[abl_i];
    abl_in.env_sugar_level = A.in.env_sugar_level[abl_i];
    abl_in.max_env_sugar_level = A.in.max_env_sugar_level[abl_i];
    abl_out.agent_id = A.out.agent_id[abl_i];
    abl_out.state = A.out.state[abl_i];
    abl_out.sugar_level = A.out.sugar_level[abl_i];
    abl_out.metabolism = A.out.metabolism[abl_i];
    movement_transaction(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.agent_id[abl_i] = abl_out.agent_id;
    A.out.state[abl_i] = abl_out.state;
    A.out.sugar_level[abl_i] = abl_out.sugar_level;
    A.out.metabolism[abl_i] = abl_out.metabolism;
}
static int abl_launch_movement_transaction(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_movement_transaction A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.pos = (float2 *) L->in_cols[0];
    A.out.pos = (float2 *) L->out_cols[0];
    A.in.target_pos = (float2 *) L->in_cols[1];
    A.out.target_pos = (float2 *) L->out_cols[1];
    A.in.agent_id = (int *) L->in_cols[2];
    A.out.agent_id = (int *) L->out_cols[2];
    A.in.state = (int *) L->in_cols[3];
    A.out.state = (int *) L->out_cols[3];
    A.in.sugar_level = (int *) L->in_cols[4];
    A.out.sugar_level = (int *) L->out_cols[4];
    A.in.metabolism = (int *) L->in_cols[5];
    A.out.metabolism = (int *) L->out_cols[5];
    A.in.env_sugar_level = (int *) L->in_cols[6];
    A.out.env_sugar_level = (int *) L->out_cols[6];
    A.in.max_env_sugar_level = (int *) L->in_cols[7];
    A.out.max_env_sugar_level = (int *) L->out_cols[7];
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
    abl_kernel_movement_transaction<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
__device__ __forceinline__ void abl_ens_body_movement_transaction(const abl_ens_launch &A, long abl_vb, long abl_ts) {
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
            return !(dist_float2(abl_p, abl_p1) > abl_G.radius);
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
    Agent abl_in, abl_out;
    abl_in.pos = ((const float2 *) A.in_cols[0])[abl_i];
    abl_in.target_pos = ((const float2 *) A.in_cols[1])[abl_i];
    abl_in.agent_id = ((const int *) A.in_cols[2])[abl_i];
    abl_in.state = ((const int *) A.in_cols[3])[abl_i];
    abl_in.sugar_level = ((const int *) A.in_cols[4])[abl_i];
    abl_in.metabolism = ((const int *) A.in_cols[5])[abl_i];
    abl_in.env_sugar_level = ((const int *) A.in_cols[6])[abl_i];
    abl_in.max_env_sugar_level = ((const int *) A.in_cols[7])[abl_i];
    abl_out.agent_id = ((const int *) A.out_cols[2])[abl_i];
    abl_out.state = ((const int *) A.out_cols[3])[abl_i];
    abl_out.sugar_level = ((const int *) A.out_cols[4])[abl_i];
    abl_out.metabolism = ((const int *) A.out_cols[5])[abl_i];
    movement_transaction(abl_Gr, A.views[abl_r], abl_K, &abl_in, &abl_out);
    ((int *) A.out_cols[2])[abl_i] = abl_out.agent_id;
    ((int *) A.out_cols[3])[abl_i] = abl_out.state;
    ((int *) A.out_cols[4])[abl_i] = abl_out.sugar_level;
    ((int *) A.out_cols[5])[abl_i] = abl_out.metabolism;
}
#ifndef ABL_PERSIST
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ens_movement_transaction(const __grid_constant__ abl_ens_launch A) {
    abl_ens_body_movement_transaction(A, blockIdx.x, A.timestep);
}
static int abl_launch_ens_movement_transaction(const abl_ens_launch *L, cudaStream_t abl_stream) {
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (L->n + abl_block - 1) / abl_block;
    abl_kernel_ens_movement_transaction<<<abl_grid, abl_block, L->smem, abl_stream>>>(*L);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
#ifndef ABL_PERSIST
static double abl_radius_movement_transaction(const void *abl_gp) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    return (double) (abl_G.radius);
}
#endif

__host__ __device__ static inline int calc_max_env_sugar_level(const abl_globals &abl_G, abl::rng &abl_R, int x, int y) {
    int gmax = abl_G.global_max_env_sugar_level;
    float2 pos = float2_create(x, y);
    int max = 0;
    double d1 = dist_float2(pos, abl_G.sugar_center1);
    max += ((float) gmax * exp((((-d1) * d1) / (2.0 * abl_G.sugar_variance))));
    double d2 = dist_float2(pos, abl_G.sugar_center2);
    max += ((float) gmax * exp((((-d2) * d2) / (2.0 * abl_G.sugar_variance))));
    return max;
}

#ifndef ABL_PERSIST
extern "C" int abl_persist_launch_sugarscape(const void *, int *, int, size_t, int *, cudaStream_t);
static const abl_member_desc abl_members_Agent[] = {
    {"pos", ABL_T_FLOAT2, 2, 8, 1},
    {"target_pos", ABL_T_FLOAT2, 2, 8, 0},
    {"agent_id", ABL_T_INT, 1, 4, 0},
    {"state", ABL_T_INT, 1, 4, 0},
    {"sugar_level", ABL_T_INT, 1, 4, 0},
    {"metabolism", ABL_T_INT, 1, 4, 0},
    {"env_sugar_level", ABL_T_INT, 1, 4, 0},
    {"max_env_sugar_level", ABL_T_INT, 1, 4, 0},
};
static const abl_agent_desc abl_agents[] = {
    {"Agent", 8, abl_members_Agent, 0, 2},
};
static const abl_global_desc abl_global_table[] = {
    {"PI", ABL_T_FLOAT, offsetof(abl_globals, PI)},
    {"AGENT_STATE_UNOCCUPIED", ABL_T_INT, offsetof(abl_globals, AGENT_STATE_UNOCCUPIED)},
    {"AGENT_STATE_OCCUPIED", ABL_T_INT, offsetof(abl_globals, AGENT_STATE_OCCUPIED)},
    {"AGENT_STATE_MOVEMENT_REQUESTED", ABL_T_INT, offsetof(abl_globals, AGENT_STATE_MOVEMENT_REQUESTED)},
    {"AGENT_STATE_MOVEMENT_UNRESOLVED", ABL_T_INT, offsetof(abl_globals, AGENT_STATE_MOVEMENT_UNRESOLVED)},
    {"SUGAR_GROWBACK_RATE", ABL_T_INT, offsetof(abl_globals, SUGAR_GROWBACK_RATE)},
    {"min_start_sugar_level", ABL_T_INT, offsetof(abl_globals, min_start_sugar_level)},
    {"max_start_sugar_level", ABL_T_INT, offsetof(abl_globals, max_start_sugar_level)},
    {"radius", ABL_T_FLOAT, offsetof(abl_globals, radius)},
    {"num_timesteps", ABL_T_INT, offsetof(abl_globals, num_timesteps)},
    {"occupiedFrac", ABL_T_FLOAT, offsetof(abl_globals, occupiedFrac)},
    {"num_agents", ABL_T_INT, offsetof(abl_globals, num_agents)},
    {"grid_width", ABL_T_INT, offsetof(abl_globals, grid_width)},
    {"sugar_center1", ABL_T_FLOAT2, offsetof(abl_globals, sugar_center1)},
    {"sugar_center2", ABL_T_FLOAT2, offsetof(abl_globals, sugar_center2)},
    {"global_max_env_sugar_level", ABL_T_INT, offsetof(abl_globals, global_max_env_sugar_level)},
    {"sugar_variance", ABL_T_FLOAT, offsetof(abl_globals, sugar_variance)},
    {nullptr, 0, 0}
};
static void abl_env_bounds(const void *abl_gp, double *abl_min, double *abl_max) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    float2 abl_lo = float2_fill(0);
    float2 abl_hi = float2_fill(abl_G.grid_width);
    abl_min[0] = abl_lo.x; abl_min[1] = abl_lo.y; abl_min[2] = 0;
    abl_max[0] = abl_hi.x; abl_max[1] = abl_hi.y; abl_max[2] = 0;
}
static const abl_step_desc abl_steps[] = {
    {"metabolise_and_growback", 0, -1, 1, nullptr, 0u, 64u, abl_launch_metabolise_and_growback, 0, -1, 0, abl_launch_ens_metabolise_and_growback, 0, 0, 124u, 0},
    {"movement_request", 0, 0, 1, abl_radius_movement_request, 73u, 0u, abl_launch_movement_request, 0, -1, 0, abl_launch_ens_movement_request, 0, 1, 10u, 1},
    {"movement_response", 0, 0, 1, abl_radius_movement_response, 63u, 0u, abl_launch_movement_response, 0, -1, 0, abl_launch_ens_movement_response, 0, 1, 60u, 1},
    {"movement_transaction", 0, 0, 1, abl_radius_movement_transaction, 13u, 0u, abl_launch_movement_transaction, 0, -1, 0, abl_launch_ens_movement_transaction, 0, 1, 60u, 1},
};
static const abl_step_desc abl_steps_ordered[] = {
    abl_steps[0],
    abl_steps[1],
    abl_steps[2],
    abl_steps[3],
    {nullptr, 0, -1, 0, nullptr, 0u, 0u, nullptr, 0, -1, 0, nullptr, 0}
};
extern const abl_model_desc abl_desc = {
    "sugarscape", 1, abl_agents, 4, abl_steps_ordered, sizeof(abl_globals), &abl_globals_default, 17, abl_global_table, 2, abl_env_bounds, nullptr, 0, nullptr, abl_persist_launch_sugarscape
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
        size_t n = agents.agents_Agent.len;
        const Agent *aos = (const Agent *) agents.agents_Agent.values;
        float2 *c0 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c0[i] = aos[i].pos;
        float2 *c1 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c1[i] = aos[i].target_pos;
        int *c2 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c2[i] = aos[i].agent_id;
        int *c3 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c3[i] = aos[i].state;
        int *c4 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c4[i] = aos[i].sugar_level;
        int *c5 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c5[i] = aos[i].metabolism;
        int *c6 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c6[i] = aos[i].env_sugar_level;
        int *c7 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c7[i] = aos[i].max_env_sugar_level;
        const void *cols[] = {c0, c1, c2, c3, c4, c5, c6, c7};
        abl_check(abl_upload(ctx, 0, cols, n), "abl_upload");
        std::free(c0);
        std::free(c1);
        std::free(c2);
        std::free(c3);
        std::free(c4);
        std::free(c5);
        std::free(c6);
        std::free(c7);
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
        int *c2 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        int *c3 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        int *c4 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        int *c5 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        int *c6 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        int *c7 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        void *cols[] = {c0, c1, c2, c3, c4, c5, c6, c7};
        size_t cap = n;
        abl_check(abl_download(ctx, 0, cols, &cap), "abl_download");
        dyn_array_clean(&agents.agents_Agent);
        agents.agents_Agent = dyn_array_create_fixed(sizeof(Agent), n);
        Agent *aos = (Agent *) agents.agents_Agent.values;
        for (size_t i = 0; i < n; i++) {
            aos[i].pos = c0[i];
            aos[i].target_pos = c1[i];
            aos[i].agent_id = c2[i];
            aos[i].state = c3[i];
            aos[i].sugar_level = c4[i];
            aos[i].metabolism = c5[i];
            aos[i].env_sugar_level = c6[i];
            aos[i].max_env_sugar_level = c7[i];
        }
        std::free(c0);
        std::free(c1);
        std::free(c2);
        std::free(c3);
        std::free(c4);
        std::free(c5);
        std::free(c6);
        std::free(c7);
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
    int id = 0;
    for (int x = 0, _var0 = abl_G.grid_width; x < _var0; ++x) {
        for (int y = 0, _var1 = abl_G.grid_width; y < _var1; ++y) {
            bool occupied = (random_3(abl_G, abl_R, 1.0) < abl_G.occupiedFrac);
            int max_env_sugar_level = calc_max_env_sugar_level(abl_G, abl_R, x, y);
            *DYN_ARRAY_PLACE(&agents.agents_Agent, Agent) = ([&]() { Agent abl_a; abl_a.pos = float2_create(((float) x + 0.5), ((float) y + 0.5)); abl_a.target_pos = float2_fill(0); abl_a.agent_id = id; abl_a.state = (occupied ? abl_G.AGENT_STATE_OCCUPIED : abl_G.AGENT_STATE_UNOCCUPIED); abl_a.sugar_level = (occupied ? abl_random_int(abl_R, abl_G.min_start_sugar_level, abl_G.max_start_sugar_level) : 0); abl_a.metabolism = (occupied ? 1 : 0); abl_a.env_sugar_level = abl_random_int(abl_R, 0, max_env_sugar_level); abl_a.max_env_sugar_level = max_env_sugar_level; return abl_a; }());
            id += 1;
        }
    }
    abl_simulate(abl_G.num_timesteps);
    return 0;
}
#else
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_PERSIST_MIN_BLOCKS) abl_kernel_ens_persist(const abl::persist_prog *abl_P, int *abl_err) {
    abl::persist_run<abl_float, 2>(abl_P, abl_err, [&](const abl_ens_launch &abl_L, long abl_vb, long abl_ts) {
        switch (abl_L.step_index) {
            case 0: abl_ens_body_metabolise_and_growback(abl_L, abl_vb, abl_ts); break;
            case 1: abl_ens_body_movement_request(abl_L, abl_vb, abl_ts); break;
            case 2: abl_ens_body_movement_response(abl_L, abl_vb, abl_ts); break;
            case 3: abl_ens_body_movement_transaction(abl_L, abl_vb, abl_ts); break;
            default: break;
        }
    });
}
#endif

}  // namespace abl_model_sugarscape

#ifdef ABL_PERSIST
extern "C" int abl_persist_launch_sugarscape(const void *abl_prog, int *abl_err, int abl_block, size_t abl_smem, int *abl_grid, cudaStream_t abl_stream) {
    return abl::persist_launch((const void *) abl_model_sugarscape::abl_kernel_ens_persist, abl_prog, abl_err, abl_block, abl_smem, abl_grid, abl_stream);
}
#endif
#ifndef ABL_PERSIST
extern "C" const abl_model_desc *abl_model_desc_sugarscape(void) {
    return &abl_model_sugarscape::abl_desc;
}
#endif

#if defined(ABL_STANDALONE_MAIN) && !defined(ABL_PERSIST)
extern "C" const abl_model_desc *const abl_builtin_models[] = {
    &abl_model_sugarscape::abl_desc, nullptr};
int main() { return abl_model_sugarscape::abl_main(); }
#endif
