// Generated by OpenABL -b cuda (model "grazers").
#include "abl_gen.cuh"

namespace abl_model_grazers {

typedef double abl_float;
#include "abl_math.cuh"

typedef struct {
    float2 pos;
    float2 dir;
    double fed;
} Grazer;
static const type_info Grazer_info[] = {
    { TYPE_FLOAT2, offsetof(Grazer, pos), "pos", true },
    { TYPE_FLOAT2, offsetof(Grazer, dir), "dir", false },
    { TYPE_FLOAT, offsetof(Grazer, fed), "fed", false },
    { TYPE_END, sizeof(Grazer), NULL }
};

typedef struct {
    float2 pos;
    double grass;
} Patch;
static const type_info Patch_info[] = {
    { TYPE_FLOAT2, offsetof(Patch, pos), "pos", true },
    { TYPE_FLOAT, offsetof(Patch, grass), "grass", false },
    { TYPE_END, sizeof(Patch), NULL }
};

struct agent_struct {
    dyn_array agents_Grazer;
    dyn_array agents_Grazer_dbuf;
    dyn_array agents_Patch;
    dyn_array agents_Patch_dbuf;
};
static struct agent_struct agents;
static const agent_info agents_info[] = {
    { Grazer_info, offsetof(struct agent_struct, agents_Grazer), "Grazer" },
    { Patch_info, offsetof(struct agent_struct, agents_Patch), "Patch" },
    { NULL, 0, NULL }
};

struct abl_globals {
    double PI;
    int num_timesteps;
    int num_agents;
    double W;
    double reach;
};
static const abl_globals abl_globals_default = {
    3.14159,
    40,
    2000,
    40.0,
    1.5,
};
static abl_globals abl_G = abl_globals_default;
static abl::rng abl_R;  // unused on the host: main() draws from the host stream
struct abl_cols_Grazer {
    float2 *pos;
    float2 *dir;
    double *fed;
};
struct abl_cols_Patch {
    float2 *pos;
    double *grass;
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
__device__ static void graze(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Grazer* in, Grazer* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    double food = 0.0;
    float2 pull = float2_create(0, 0);
    {
        const abl::near_query<2> abl_q1(abl_NB, (double) in->pos.x, (double) in->pos.y, 0.0, abl_K.self);
        abl::near_list_cursor<2> abl_c1(abl_NB, abl_q1, abl_K);
        auto abl_exact1 = [&](int abl_s) -> bool {
            const float2 abl_p = ((const float2 *) abl_NB.cols[0])[abl_s];
            return !(dist_float2(abl_p, in->pos) > abl_G.reach);
        };
        while (abl_c1.fill(abl_q1, abl_exact1)) {
            int abl_pslot1 = abl_c1.slot(0);
            Patch abl_pnx1;
            abl_pnx1.pos = ((const float2 *) abl_NB.cols[0])[abl_pslot1];
            abl_pnx1.grass = ((const double *) abl_NB.cols[1])[abl_pslot1];
            for (int abl_k = 0; abl_k < abl_c1.cnt; ++abl_k) {
                const int abl_slot1 = abl_pslot1;
                Patch abl_nx1 = abl_pnx1;
                if (abl_k + 1 < abl_c1.cnt) {
                    abl_pslot1 = abl_c1.slot(abl_k + 1);
                    abl_pnx1.pos = ((const float2 *) abl_NB.cols[0])[abl_pslot1];
                    abl_pnx1.grass = ((const double *) abl_NB.cols[1])[abl_pslot1];
                }
                Patch* p = &abl_nx1;
                {
                    food += p->grass;
                    pull = float2_add(pull, float2_mul_scalar(float2_sub(p->pos, in->pos), p->grass));
                }
            }
        }
    }
    float2 d = float2_add(in->dir, float2_mul_scalar(pull, 0.01));
    double len = length_float2(d);
    if ((len > 0)) {
        d = float2_div_scalar(d, len);
    }
    out->dir = d;
    out->pos = wraparound_1(abl_G, abl_R, float2_add(in->pos, float2_mul_scalar(d, 0.2)), float2_fill(abl_G.W));
    out->fed = ((in->fed * 0.9) + food);
}

#ifndef ABL_PERSIST
struct abl_kargs_graze {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Grazer in, out;
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
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_graze(const __grid_constant__ abl_kargs_graze A) {
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
            return !(dist_float2(abl_p, abl_p1) > abl_G.reach);
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
    Grazer abl_in, abl_out;
    abl_in.pos = A.in.pos[abl_i];
    abl_in.dir = A.in.dir[abl_i];
    abl_in.fed = A.in.fed[abl_i];
    graze(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.pos[abl_i] = abl_out.pos;
    A.out.dir[abl_i] = abl_out.dir;
    A.out.fed[abl_i] = abl_out.fed;
}
static int abl_launch_graze(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_graze A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.pos = (float2 *) L->in_cols[0];
    A.out.pos = (float2 *) L->out_cols[0];
    A.in.dir = (float2 *) L->in_cols[1];
    A.out.dir = (float2 *) L->out_cols[1];
    A.in.fed = (double *) L->in_cols[2];
    A.out.fed = (double *) L->out_cols[2];
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
    abl_kernel_graze<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
__device__ __forceinline__ void abl_ens_body_graze(const abl_ens_launch &A, long abl_vb, long abl_ts) {
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
            return !(dist_float2(abl_p, abl_p1) > abl_G.reach);
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
    Grazer abl_in, abl_out;
    abl_in.pos = ((const float2 *) A.in_cols[0])[abl_i];
    abl_in.dir = ((const float2 *) A.in_cols[1])[abl_i];
    abl_in.fed = ((const double *) A.in_cols[2])[abl_i];
    graze(abl_Gr, A.views[abl_r], abl_K, &abl_in, &abl_out);
    ((float2 *) A.out_cols[0])[abl_i] = abl_out.pos;
    ((float2 *) A.out_cols[1])[abl_i] = abl_out.dir;
    ((double *) A.out_cols[2])[abl_i] = abl_out.fed;
}
#ifndef ABL_PERSIST
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ens_graze(const __grid_constant__ abl_ens_launch A) {
    abl_ens_body_graze(A, blockIdx.x, A.timestep);
}
static int abl_launch_ens_graze(const abl_ens_launch *L, cudaStream_t abl_stream) {
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (L->n + abl_block - 1) / abl_block;
    abl_kernel_ens_graze<<<abl_grid, abl_block, L->smem, abl_stream>>>(*L);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
#ifndef ABL_PERSIST
static double abl_radius_graze(const void *abl_gp) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    return (double) (abl_G.reach);
}
#endif


#ifndef ABL_PERSIST
extern "C" int abl_persist_launch_grazers(const void *, int *, int, size_t, int *, cudaStream_t);
static const abl_member_desc abl_members_Grazer[] = {
    {"pos", ABL_T_FLOAT2, 2, 8, 1},
    {"dir", ABL_T_FLOAT2, 2, 8, 0},
    {"fed", ABL_T_FLOAT, 1, 8, 0},
};
static const abl_member_desc abl_members_Patch[] = {
    {"pos", ABL_T_FLOAT2, 2, 8, 1},
    {"grass", ABL_T_FLOAT, 1, 8, 0},
};
static const abl_agent_desc abl_agents[] = {
    {"Grazer", 3, abl_members_Grazer, 0, 2},
    {"Patch", 2, abl_members_Patch, 0, 2},
};
static const abl_global_desc abl_global_table[] = {
    {"PI", ABL_T_FLOAT, offsetof(abl_globals, PI)},
    {"num_timesteps", ABL_T_INT, offsetof(abl_globals, num_timesteps)},
    {"num_agents", ABL_T_INT, offsetof(abl_globals, num_agents)},
    {"W", ABL_T_FLOAT, offsetof(abl_globals, W)},
    {"reach", ABL_T_FLOAT, offsetof(abl_globals, reach)},
    {nullptr, 0, 0}
};
static void abl_env_bounds(const void *abl_gp, double *abl_min, double *abl_max) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    float2 abl_lo = float2_fill(0);
    float2 abl_hi = float2_fill(abl_G.W);
    abl_min[0] = abl_lo.x; abl_min[1] = abl_lo.y; abl_min[2] = 0;
    abl_max[0] = abl_hi.x; abl_max[1] = abl_hi.y; abl_max[2] = 0;
}
static const abl_step_desc abl_steps[] = {
    {"graze", 0, 1, 1, abl_radius_graze, 3u, 7u, abl_launch_graze, 0, -1, 0, abl_launch_ens_graze, 0, 1, 7u, 1},
};
static const abl_step_desc abl_steps_ordered[] = {
    abl_steps[0],
    {nullptr, 0, -1, 0, nullptr, 0u, 0u, nullptr, 0, -1, 0, nullptr, 0}
};
extern const abl_model_desc abl_desc = {
    "grazers", 2, abl_agents, 1, abl_steps_ordered, sizeof(abl_globals), &abl_globals_default, 5, abl_global_table, 2, abl_env_bounds, nullptr, 0, nullptr, abl_persist_launch_grazers
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
        size_t n = agents.agents_Grazer.len;
        const Grazer *aos = (const Grazer *) agents.agents_Grazer.values;
        float2 *c0 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c0[i] = aos[i].pos;
        float2 *c1 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c1[i] = aos[i].dir;
        double *c2 = (double *) std::malloc(sizeof(double) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c2[i] = aos[i].fed;
        const void *cols[] = {c0, c1, c2};
        abl_check(abl_upload(ctx, 0, cols, n), "abl_upload");
        std::free(c0);
        std::free(c1);
        std::free(c2);
    }
    {
        size_t n = agents.agents_Patch.len;
        const Patch *aos = (const Patch *) agents.agents_Patch.values;
        float2 *c0 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c0[i] = aos[i].pos;
        double *c1 = (double *) std::malloc(sizeof(double) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c1[i] = aos[i].grass;
        const void *cols[] = {c0, c1};
        abl_check(abl_upload(ctx, 1, cols, n), "abl_upload");
        std::free(c0);
        std::free(c1);
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
        void *cols[] = {c0, c1, c2};
        size_t cap = n;
        abl_check(abl_download(ctx, 0, cols, &cap), "abl_download");
        dyn_array_clean(&agents.agents_Grazer);
        agents.agents_Grazer = dyn_array_create_fixed(sizeof(Grazer), n);
        Grazer *aos = (Grazer *) agents.agents_Grazer.values;
        for (size_t i = 0; i < n; i++) {
            aos[i].pos = c0[i];
            aos[i].dir = c1[i];
            aos[i].fed = c2[i];
        }
        std::free(c0);
        std::free(c1);
        std::free(c2);
    }
    {
        size_t n = 0;
        abl_check(abl_count(ctx, 1, &n), "abl_count");
        float2 *c0 = (float2 *) std::malloc(sizeof(float2) * (n ? n : 1));
        double *c1 = (double *) std::malloc(sizeof(double) * (n ? n : 1));
        void *cols[] = {c0, c1};
        size_t cap = n;
        abl_check(abl_download(ctx, 1, cols, &cap), "abl_download");
        dyn_array_clean(&agents.agents_Patch);
        agents.agents_Patch = dyn_array_create_fixed(sizeof(Patch), n);
        Patch *aos = (Patch *) agents.agents_Patch.values;
        for (size_t i = 0; i < n; i++) {
            aos[i].pos = c0[i];
            aos[i].grass = c1[i];
        }
        std::free(c0);
        std::free(c1);
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
    for (int i = 0, _var0 = abl_G.num_agents; i < _var0; ++i) {
        *DYN_ARRAY_PLACE(&agents.agents_Grazer, Grazer) = ([&]() { Grazer abl_a; abl_a.pos = random_4(abl_G, abl_R, float2_fill(abl_G.W)); abl_a.dir = float2_create(1, 0); abl_a.fed = 0.0; return abl_a; }());
    }
    for (int i = 0, _var1 = abl_G.num_agents; i < _var1; ++i) {
        *DYN_ARRAY_PLACE(&agents.agents_Patch, Patch) = ([&]() { Patch abl_a; abl_a.pos = random_4(abl_G, abl_R, float2_fill(abl_G.W)); abl_a.grass = abl_random(abl_R, 0.0, 1.0); return abl_a; }());
    }
    abl_simulate(abl_G.num_timesteps);
    save(&agents, agents_info, "grazers.json", SAVE_JSON);
    return 0;
}
#else
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_PERSIST_MIN_BLOCKS) abl_kernel_ens_persist(const abl::persist_prog *abl_P, int *abl_err) {
    abl::persist_run<abl_float, 2>(abl_P, abl_err, [&](const abl_ens_launch &abl_L, long abl_vb, long abl_ts) {
        switch (abl_L.step_index) {
            case 0: abl_ens_body_graze(abl_L, abl_vb, abl_ts); break;
            default: break;
        }
    });
}
#endif

}  // namespace abl_model_grazers

#ifdef ABL_PERSIST
extern "C" int abl_persist_launch_grazers(const void *abl_prog, int *abl_err, int abl_block, size_t abl_smem, int *abl_grid, cudaStream_t abl_stream) {
    return abl::persist_launch((const void *) abl_model_grazers::abl_kernel_ens_persist, abl_prog, abl_err, abl_block, abl_smem, abl_grid, abl_stream);
}
#endif
#ifndef ABL_PERSIST
extern "C" const abl_model_desc *abl_model_desc_grazers(void) {
    return &abl_model_grazers::abl_desc;
}
#endif

#if defined(ABL_STANDALONE_MAIN) && !defined(ABL_PERSIST)
extern "C" const abl_model_desc *const abl_builtin_models[] = {
    &abl_model_grazers::abl_desc, nullptr};
int main() { return abl_model_grazers::abl_main(); }
#endif
