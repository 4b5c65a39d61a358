// Generated by OpenABL -b cuda (model "keratinocyte").
#include "abl_gen.cuh"

namespace abl_model_keratinocyte {

typedef double abl_float;
#include "abl_math.cuh"

typedef struct {
    int type;
    float3 pos;
    float3 force;
    int num_xy_bonds;
    int num_z_bonds;
    int num_stem_bonds;
    int cycle;
    double diff_noise_factor;
    int dead_ticks;
    int contact_inhibited_ticks;
    double motility;
    double dir;
    double movement;
} Keratinocyte;
static const type_info Keratinocyte_info[] = {
    { TYPE_INT, offsetof(Keratinocyte, type), "type", false },
    { TYPE_FLOAT3, offsetof(Keratinocyte, pos), "pos", true },
    { TYPE_FLOAT3, offsetof(Keratinocyte, force), "force", false },
    { TYPE_INT, offsetof(Keratinocyte, num_xy_bonds), "num_xy_bonds", false },
    { TYPE_INT, offsetof(Keratinocyte, num_z_bonds), "num_z_bonds", false },
    { TYPE_INT, offsetof(Keratinocyte, num_stem_bonds), "num_stem_bonds", false },
    { TYPE_INT, offsetof(Keratinocyte, cycle), "cycle", false },
    { TYPE_FLOAT, offsetof(Keratinocyte, diff_noise_factor), "diff_noise_factor", false },
    { TYPE_INT, offsetof(Keratinocyte, dead_ticks), "dead_ticks", false },
    { TYPE_INT, offsetof(Keratinocyte, contact_inhibited_ticks), "contact_inhibited_ticks", false },
    { TYPE_FLOAT, offsetof(Keratinocyte, motility), "motility", false },
    { TYPE_FLOAT, offsetof(Keratinocyte, dir), "dir", false },
    { TYPE_FLOAT, offsetof(Keratinocyte, movement), "movement", false },
    { TYPE_END, sizeof(Keratinocyte), NULL }
};

struct agent_struct {
    dyn_array agents_Keratinocyte;
    dyn_array agents_Keratinocyte_dbuf;
};
static struct agent_struct agents;
static const agent_info agents_info[] = {
    { Keratinocyte_info, offsetof(struct agent_struct, agents_Keratinocyte), "Keratinocyte" },
    { NULL, 0, NULL }
};

struct abl_globals {
    double PI;
    double K_WIDTH;
    double FORCE_IRADIUS;
    double BASEMENT_MAX_Z;
    int MAX_TO_G0_CONTACT_INHIBITED_TICKS;
    int MAX_DEAD_TICKS;
    int MAX_NUM_LATERAL_BONDS;
    int CYCLE_LENGTH[5];
    double FORCE_REP;
    double FORCE_DAMPENER;
    float SUBSTRATE_FORCE[5];
    float DOWNWARD_FORCE[5];
    float FORCE_MATRIX[25];
    double calcium_level;
    int K_TYPE_STEM;
    int K_TYPE_TA;
    int K_TYPE_COMM;
    int K_TYPE_CORN;
    int K_TYPE_HACAT;
    int num_agents;
    int num_timesteps;
    double SURFACE_WIDTH;
};
static const abl_globals abl_globals_default = {
    3.14159,
    20.0,
    10.0,
    5.0,
    300,
    600,
    4,
    { 120, 60, 0, 0, 120 },
    0.5,
    0.4,
    { 0.3, 0.1, 0.2, 0.1, 0.3 },
    { 0.1, 0.6, 0.3, 0.6, 0.1 },
    { 0.06, 0.01, 0.01, 0.01, 0.0, 0.01, 0.01, 0.01, 0.01, 0.0, 0.01, 0.01, 0.06, 0.01, 0.0, 0.01, 0.01, 0.01, 0.08, 0.0, 0.01, 0.01, 0.01, 0.08, 0.0 },
    1.3,
    0,
    1,
    2,
    3,
    4,
    100,
    100,
    500.0,
};
static abl_globals abl_G = abl_globals_default;
static abl::rng abl_R;  // unused on the host: main() draws from the host stream
struct abl_cols_Keratinocyte {
    int *type;
    float3 *pos;
    float3 *force;
    int *num_xy_bonds;
    int *num_z_bonds;
    int *num_stem_bonds;
    int *cycle;
    double *diff_noise_factor;
    int *dead_ticks;
    int *contact_inhibited_ticks;
    double *motility;
    double *dir;
    double *movement;
};
__device__ static void abl_add_Keratinocyte(abl::step_ctx &K, const Keratinocyte &c) {
    K.added = 1;
    ((int *) K.child_cols[0])[K.self] = c.type;
    ((float3 *) K.child_cols[1])[K.self] = c.pos;
    ((float3 *) K.child_cols[2])[K.self] = c.force;
    ((int *) K.child_cols[3])[K.self] = c.num_xy_bonds;
    ((int *) K.child_cols[4])[K.self] = c.num_z_bonds;
    ((int *) K.child_cols[5])[K.self] = c.num_stem_bonds;
    ((int *) K.child_cols[6])[K.self] = c.cycle;
    ((double *) K.child_cols[7])[K.self] = c.diff_noise_factor;
    ((int *) K.child_cols[8])[K.self] = c.dead_ticks;
    ((int *) K.child_cols[9])[K.self] = c.contact_inhibited_ticks;
    ((double *) K.child_cols[10])[K.self] = c.motility;
    ((double *) K.child_cols[11])[K.self] = c.dir;
    ((double *) K.child_cols[12])[K.self] = c.movement;
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
__host__ __device__ static inline bool on_substrate_surface(const abl_globals &abl_G, abl::rng &abl_R, double z) {
    return (z < abl_G.BASEMENT_MAX_Z);
}
__host__ __device__ static inline double get_ta_to_comm_diff_minor_axis(const abl_globals &abl_G, abl::rng &abl_R, double calcium_level) {
    return (abl_G.K_WIDTH * 1.5);
}
__host__ __device__ static inline double get_ta_to_comm_diff_major_axis(const abl_globals &abl_G, abl::rng &abl_R, double calcium_level) {
    return (abl_G.K_WIDTH * 5.0);
}
__host__ __device__ static inline int get_max_num_bonds(const abl_globals &abl_G, abl::rng &abl_R, double calcium_level) {
    return 6;
}
__host__ __device__ static inline bool can_stratify(const abl_globals &abl_G, abl::rng &abl_R, int cell_type, double calcium_level) {
    return (cell_type != abl_G.K_TYPE_HACAT);
}
__host__ __device__ static inline int get_max_stem_colony_size(const abl_globals &abl_G, abl::rng &abl_R, double calcium_level) {
    return 20;
}
__host__ __device__ static inline double get_new_motility(const abl_globals &abl_G, abl::rng &abl_R, int cell_type, double calcium_level) {
    if ((cell_type == abl_G.K_TYPE_TA)) {
        return 0.5;
    } else {
        return 0.0;
    }
}
__host__ __device__ static inline bool divide(const abl_globals &abl_G, abl::rng &abl_R, int type, int cycle) {
    return ((((type == abl_G.K_TYPE_STEM) || (type == abl_G.K_TYPE_TA)) || (type == abl_G.K_TYPE_HACAT)) && (cycle > abl_G.CYCLE_LENGTH[type]));
}
__host__ __device__ static inline double get_new_coord(const abl_globals &abl_G, abl::rng &abl_R, double old_coord, bool pos_only) {
    double coord = 0.0;
    while ((coord == 0)) {
        coord = abl_random(abl_R, 0, (abl_G.K_WIDTH / 10.0));
    }
    if (((!pos_only) && (coord > 0.5))) {
        coord = (-coord);
    }
    return (old_coord + coord);
}
__host__ __device__ static inline int start_new_cycle_position(const abl_globals &abl_G, abl::rng &abl_R, int type) {
    double cycle_fraction = (float) (abl_G.CYCLE_LENGTH[type] / 4);
    double pos = abl_random(abl_R, 0, cycle_fraction);
    return (int) round(pos);
}
__host__ __device__ static inline double ellipse_radius(const abl_globals &abl_G, abl::rng &abl_R, double major_radius, double minor_radius, double theta) {
    double a_squ = (major_radius * major_radius);
    double b_squ = (minor_radius * minor_radius);
    double sin_theta = sin(theta);
    double sin_theta_squ = (sin_theta * sin_theta);
    double cos_theta = cos(theta);
    double cos_theta_squ = (cos_theta * cos_theta);
    double r_squ = ((a_squ * b_squ) / ((a_squ * sin_theta_squ) + (b_squ * cos_theta_squ)));
    double r = sqrt(r_squ);
    return r;
}
__host__ __device__ static inline bool check_distance(const abl_globals &abl_G, abl::rng &abl_R, double nearest_dist, double nearest_xy, double nearest_z, double major_radius, double minor_radius, double thres) {
    if ((nearest_dist == (-1))) {
        return true;
    }
    double theta = tan((nearest_z / nearest_xy));
    double er = ellipse_radius(abl_G, abl_R, major_radius, minor_radius, theta);
    return ((thres * er) < nearest_dist);
}
__host__ __device__ static inline bool on_colony_edge(const abl_globals &abl_G, abl::rng &abl_R, int num_bonds) {
    return (num_bonds <= 2);
}
__device__ static void cycle(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Keratinocyte* in, Keratinocyte* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    int contacts = (in->num_xy_bonds + in->num_z_bonds);
    if (((in->pos.x == 0) || (in->pos.x == abl_G.SURFACE_WIDTH))) {
        contacts += 2;
    }
    if (((in->pos.y == 0) || (in->pos.y == abl_G.SURFACE_WIDTH))) {
        contacts += 2;
    }
    if ((contacts <= get_max_num_bonds(abl_G, abl_R, abl_G.calcium_level))) {
        out->cycle = (in->cycle + 1);
        out->contact_inhibited_ticks = 0;
    } else {
        out->contact_inhibited_ticks = (in->contact_inhibited_ticks + 1);
    }
    if (divide(abl_G, abl_R, in->type, in->cycle)) {
        int new_cycle = start_new_cycle_position(abl_G, abl_R, in->type);
        float3 new_pos = ([&]() { const auto abl_e3_2 = in->pos.z; const auto abl_e3_1 = get_new_coord(abl_G, abl_R, in->pos.y, false); const auto abl_e3_0 = get_new_coord(abl_G, abl_R, in->pos.x, false); return float3_create(abl_e3_0, abl_e3_1, abl_e3_2); }());
        double new_diff_noise_factor = abl_random(abl_R, 0.9, 1.1);
        double new_dir = random_3(abl_G, abl_R, (2.0 * abl_G.PI));
        double new_motility = (abl_random(abl_R, 0.5, 1.0) * get_new_motility(abl_G, abl_R, in->type, abl_G.calcium_level));
        if ((can_stratify(abl_G, abl_R, in->type, abl_G.calcium_level) && (in->num_xy_bonds >= abl_G.MAX_NUM_LATERAL_BONDS))) {
            new_pos.z = get_new_coord(abl_G, abl_R, in->pos.z, true);
        }
        out->cycle = start_new_cycle_position(abl_G, abl_R, in->type);
        abl_add_Keratinocyte(abl_K, ([&]() { Keratinocyte abl_a; abl_a.type = in->type; abl_a.pos = new_pos; abl_a.force = float3_fill(0); abl_a.num_xy_bonds = 0; abl_a.num_z_bonds = 0; abl_a.num_stem_bonds = 0; abl_a.cycle = new_cycle; abl_a.diff_noise_factor = new_diff_noise_factor; abl_a.dead_ticks = 0; abl_a.contact_inhibited_ticks = 0; abl_a.motility = new_motility; abl_a.dir = new_dir; abl_a.movement = 0.0; return abl_a; }()));
    }
}

#ifndef ABL_PERSIST
struct abl_kargs_cycle {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Keratinocyte in, out;
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
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_cycle(const __grid_constant__ abl_kargs_cycle A) {
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
    Keratinocyte abl_in, abl_out;
    abl_in.type = A.in.type[abl_i];
    abl_in.pos = A.in.pos[abl_i];
    abl_in.force = A.in.force[abl_i];
    abl_in.num_xy_bonds = A.in.num_xy_bonds[abl_i];
    abl_in.num_z_bonds = A.in.num_z_bonds[abl_i];
    abl_in.num_stem_bonds = A.in.num_stem_bonds[abl_i];
    abl_in.cycle = A.in.cycle[abl_i];
    abl_in.diff_noise_factor = A.in.diff_noise_factor[abl_i];
    abl_in.dead_ticks = A.in.dead_ticks[abl_i];
    abl_in.contact_inhibited_ticks = A.in.contact_inhibited_ticks[abl_i];
    abl_in.motility = A.in.motility[abl_i];
    abl_in.dir = A.in.dir[abl_i];
    abl_in.movement = A.in.movement[abl_i];
    abl_out = abl_in;
    cycle(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.type[abl_i] = abl_out.type;
    A.out.pos[abl_i] = abl_out.pos;
    A.out.force[abl_i] = abl_out.force;
    A.out.num_xy_bonds[abl_i] = abl_out.num_xy_bonds;
    A.out.num_z_bonds[abl_i] = abl_out.num_z_bonds;
    A.out.num_stem_bonds[abl_i] = abl_out.num_stem_bonds;
    A.out.cycle[abl_i] = abl_out.cycle;
    A.out.diff_noise_factor[abl_i] = abl_out.diff_noise_factor;
    A.out.dead_ticks[abl_i] = abl_out.dead_ticks;
    A.out.contact_inhibited_ticks[abl_i] = abl_out.contact_inhibited_ticks;
    A.out.motility[abl_i] = abl_out.motility;
    A.out.dir[abl_i] = abl_out.dir;
    A.out.movement[abl_i] = abl_out.movement;
    A.child_flag[abl_i] = (uint8_t) abl_K.added;
}
static int abl_launch_cycle(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_cycle A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.type = (int *) L->in_cols[0];
    A.out.type = (int *) L->out_cols[0];
    A.in.pos = (float3 *) L->in_cols[1];
    A.out.pos = (float3 *) L->out_cols[1];
    A.in.force = (float3 *) L->in_cols[2];
    A.out.force = (float3 *) L->out_cols[2];
    A.in.num_xy_bonds = (int *) L->in_cols[3];
    A.out.num_xy_bonds = (int *) L->out_cols[3];
    A.in.num_z_bonds = (int *) L->in_cols[4];
    A.out.num_z_bonds = (int *) L->out_cols[4];
    A.in.num_stem_bonds = (int *) L->in_cols[5];
    A.out.num_stem_bonds = (int *) L->out_cols[5];
    A.in.cycle = (int *) L->in_cols[6];
    A.out.cycle = (int *) L->out_cols[6];
    A.in.diff_noise_factor = (double *) L->in_cols[7];
    A.out.diff_noise_factor = (double *) L->out_cols[7];
    A.in.dead_ticks = (int *) L->in_cols[8];
    A.out.dead_ticks = (int *) L->out_cols[8];
    A.in.contact_inhibited_ticks = (int *) L->in_cols[9];
    A.out.contact_inhibited_ticks = (int *) L->out_cols[9];
    A.in.motility = (double *) L->in_cols[10];
    A.out.motility = (double *) L->out_cols[10];
    A.in.dir = (double *) L->in_cols[11];
    A.out.dir = (double *) L->out_cols[11];
    A.in.movement = (double *) L->in_cols[12];
    A.out.movement = (double *) L->out_cols[12];
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
    abl_kernel_cycle<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif

__device__ static void differentiate(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Keratinocyte* in, Keratinocyte* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    double nearest_dist = (float) (-1);
    double nearest_xy = (float) (-1);
    double nearest_z = (float) (-1);
    int num_stem_neighbors = 0;
    double radius = 125.0;
    {
        const abl::near_query<3> abl_q1(abl_NB, (double) in->pos.x, (double) in->pos.y, (double) in->pos.z, abl_K.self);
        abl::near_list_cursor<3> abl_c1(abl_NB, abl_q1, abl_K);
        auto abl_exact1 = [&](int abl_s) -> bool {
            const float3 abl_p = ((const float3 *) abl_NB.cols[1])[abl_s];
            return !(dist_float3(abl_p, in->pos) > radius);
        };
        while (abl_c1.fill(abl_q1, abl_exact1)) {
            int abl_pslot1 = abl_c1.slot(0);
            Keratinocyte abl_pnx1;
            abl_pnx1.type = ((const int *) abl_NB.cols[0])[abl_pslot1];
            abl_pnx1.pos = ((const float3 *) abl_NB.cols[1])[abl_pslot1];
            for (int abl_k = 0; abl_k < abl_c1.cnt; ++abl_k) {
                const int abl_slot1 = abl_pslot1;
                Keratinocyte abl_nx1 = abl_pnx1;
                if (abl_k + 1 < abl_c1.cnt) {
                    abl_pslot1 = abl_c1.slot(abl_k + 1);
                    abl_pnx1.type = ((const int *) abl_NB.cols[0])[abl_pslot1];
                    abl_pnx1.pos = ((const float3 *) abl_NB.cols[1])[abl_pslot1];
                }
                Keratinocyte* other = &abl_nx1;
                {
                    if ((in->type == abl_G.K_TYPE_STEM)) {
                        if ((on_colony_edge(abl_G, abl_R, in->num_stem_bonds) && (other->type == abl_G.K_TYPE_STEM))) {
                            double dist = dist_float3(in->pos, other->pos);
                            double max_dist = ((abl_G.K_WIDTH * (float) get_max_stem_colony_size(abl_G, abl_R, abl_G.calcium_level)) / 2.0);
                            if ((dist < max_dist)) {
                                num_stem_neighbors += 1;
                            }
                        }
                    } else if ((in->type == abl_G.K_TYPE_TA)) {
                        if ((other->type == abl_G.K_TYPE_STEM)) {
                            double dist = dist_float3(in->pos, other->pos);
                            if (((nearest_dist == (-1)) || (dist < nearest_dist))) {
                                nearest_dist = dist;
                                nearest_xy = dist_float2(float2_create(in->pos.x, in->pos.y), float2_create(other->pos.x, other->pos.y));
                                nearest_z = ((in->pos.z < other->pos.z) ? (other->pos.z - in->pos.z) : (in->pos.z - other->pos.z));
                            }
                        }
                    }
                }
            }
        }
    }
    if ((in->type == abl_G.K_TYPE_STEM)) {
        if (on_colony_edge(abl_G, abl_R, in->num_stem_bonds)) {
            if ((num_stem_neighbors > get_max_stem_colony_size(abl_G, abl_R, abl_G.calcium_level))) {
                out->type = abl_G.K_TYPE_TA;
            }
        }
        if ((!on_substrate_surface(abl_G, abl_R, in->pos.z))) {
            out->type = abl_G.K_TYPE_TA;
        }
    } else if ((in->type == abl_G.K_TYPE_TA)) {
        bool do_diff = check_distance(abl_G, abl_R, nearest_dist, nearest_xy, nearest_z, get_ta_to_comm_diff_major_axis(abl_G, abl_R, abl_G.calcium_level), get_ta_to_comm_diff_minor_axis(abl_G, abl_R, abl_G.calcium_level), in->diff_noise_factor);
        if (do_diff) {
            out->type = abl_G.K_TYPE_COMM;
        } else if ((in->contact_inhibited_ticks >= abl_G.MAX_TO_G0_CONTACT_INHIBITED_TICKS)) {
            out->type = abl_G.K_TYPE_COMM;
        }
    } else if ((in->type == abl_G.K_TYPE_COMM)) {
        out->dead_ticks = (in->dead_ticks + 1);
        if (((in->dead_ticks + 1) > abl_G.MAX_DEAD_TICKS)) {
            out->type = abl_G.K_TYPE_CORN;
        }
    } else if ((in->type == abl_G.K_TYPE_HACAT)) {
        if ((in->contact_inhibited_ticks >= abl_G.MAX_TO_G0_CONTACT_INHIBITED_TICKS)) {
            out->type = abl_G.K_TYPE_COMM;
        }
    }
}

#ifndef ABL_PERSIST
struct abl_kargs_differentiate {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Keratinocyte in, out;
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
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_differentiate(const __grid_constant__ abl_kargs_differentiate A) {
    int abl_j;
    {
        const abl_globals &abl_G = A.G;
        const long abl_t1 = (long) blockIdx.x * blockDim.x + threadIdx.x;
        const bool abl_has = abl_t1 < A.n;
        const long abl_i1 = abl_has ? (A.visit ? (long) A.visit[abl_t1] : abl_t1) : 0;
        const float3 abl_p1 = abl_has ? A.in.pos[abl_i1] : float3{};
        const abl::near_query<3> abl_q0(A.NB, (double) abl_p1.x, (double) abl_p1.y, (double) abl_p1.z, abl_has ? abl_i1 : -1);
        auto abl_x0 = [&](int abl_s) -> bool {
            const float3 abl_p = ((const float3 *) A.NB.cols[1])[abl_s];
            return !(dist_float3(abl_p, abl_p1) > ((double) (125.0)));
        };
        abl_j = abl::presort_block<3>(A.NB, abl_has, abl_q0, abl_x0);
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
    Keratinocyte abl_in, abl_out;
    abl_in.type = A.in.type[abl_i];
    abl_in.pos = A.in.pos[abl_i];
    abl_in.force = A.in.force[abl_i];
    abl_in.num_xy_bonds = A.in.num_xy_bonds[abl_i];
    abl_in.num_z_bonds = A.in.num_z_bonds[abl_i];
    abl_in.num_stem_bonds = A.in.num_stem_bonds[abl_i];
    abl_in.cycle = A.in.cycle[abl_i];
    abl_in.diff_noise_factor = A.in.diff_noise_factor[abl_i];
    abl_in.dead_ticks = A.in.dead_ticks[abl_i];
    abl_in.contact_inhibited_ticks = A.in.contact_inhibited_ticks[abl_i];
    abl_in.motility = A.in.motility[abl_i];
    abl_in.dir = A.in.dir[abl_i];
    abl_in.movement = A.in.movement[abl_i];
    abl_out = abl_in;
    differentiate(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.type[abl_i] = abl_out.type;
    A.out.pos[abl_i] = abl_out.pos;
    A.out.force[abl_i] = abl_out.force;
    A.out.num_xy_bonds[abl_i] = abl_out.num_xy_bonds;
    A.out.num_z_bonds[abl_i] = abl_out.num_z_bonds;
    A.out.num_stem_bonds[abl_i] = abl_out.num_stem_bonds;
    A.out.cycle[abl_i] = abl_out.cycle;
    A.out.diff_noise_factor[abl_i] = abl_out.diff_noise_factor;
    A.out.dead_ticks[abl_i] = abl_out.dead_ticks;
    A.out.contact_inhibited_ticks[abl_i] = abl_out.contact_inhibited_ticks;
    A.out.motility[abl_i] = abl_out.motility;
    A.out.dir[abl_i] = abl_out.dir;
    A.out.movement[abl_i] = abl_out.movement;
}
static int abl_launch_differentiate(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_differentiate A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.type = (int *) L->in_cols[0];
    A.out.type = (int *) L->out_cols[0];
    A.in.pos = (float3 *) L->in_cols[1];
    A.out.pos = (float3 *) L->out_cols[1];
    A.in.force = (float3 *) L->in_cols[2];
    A.out.force = (float3 *) L->out_cols[2];
    A.in.num_xy_bonds = (int *) L->in_cols[3];
    A.out.num_xy_bonds = (int *) L->out_cols[3];
    A.in.num_z_bonds = (int *) L->in_cols[4];
    A.out.num_z_bonds = (int *) L->out_cols[4];
    A.in.num_stem_bonds = (int *) L->in_cols[5];
    A.out.num_stem_bonds = (int *) L->out_cols[5];
    A.in.cycle = (int *) L->in_cols[6];
    A.out.cycle = (int *) L->out_cols[6];
    A.in.diff_noise_factor = (double *) L->in_cols[7];
    A.out.diff_noise_factor = (double *) L->out_cols[7];
    A.in.dead_ticks = (int *) L->in_cols[8];
    A.out.dead_ticks = (int *) L->out_cols[8];
    A.in.contact_inhibited_ticks = (int *) L->in_cols[9];
    A.out.contact_inhibited_ticks = (int *) L->out_cols[9];
    A.in.motility = (double *) L->in_cols[10];
    A.out.motility = (double *) L->out_cols[10];
    A.in.dir = (double *) L->in_cols[11];
    A.out.dir = (double *) L->out_cols[11];
    A.in.movement = (double *) L->in_cols[12];
    A.out.movement = (double *) L->out_cols[12];
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
    abl_kernel_differentiate<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
__device__ __forceinline__ void abl_ens_body_differentiate(const abl_ens_launch &A, long abl_vb, long abl_ts) {
    int abl_j;
    {
        const long abl_t1 = abl_vb * blockDim.x + threadIdx.x;
        const bool abl_has = abl_t1 < A.n;
        const long abl_i1 = abl_has ? (A.visit_order ? (long) A.visit_order[abl_t1] : abl_t1) : 0;
        const int abl_r1 = abl_has ? A.replica[abl_i1] : 0;
        const abl_globals &abl_G = ((const abl_globals *) A.globals)[abl_r1];
        const abl_near_view &abl_V1 = A.views[abl_r1];
        const float3 abl_p1 = abl_has ? ((const float3 *) A.in_cols[1])[abl_i1] : float3{};
        const abl::near_query<3> abl_q0(abl_V1, (double) abl_p1.x, (double) abl_p1.y, (double) abl_p1.z, abl_has ? abl_i1 : -1);
        auto abl_x0 = [&](int abl_s) -> bool {
            const float3 abl_p = ((const float3 *) abl_V1.cols[1])[abl_s];
            return !(dist_float3(abl_p, abl_p1) > ((double) (125.0)));
        };
        abl_j = abl::presort_block<3>(abl_V1, abl_has, abl_q0, abl_x0);
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
    Keratinocyte abl_in, abl_out;
    abl_in.type = ((const int *) A.in_cols[0])[abl_i];
    abl_in.pos = ((const float3 *) A.in_cols[1])[abl_i];
    abl_in.force = ((const float3 *) A.in_cols[2])[abl_i];
    abl_in.num_xy_bonds = ((const int *) A.in_cols[3])[abl_i];
    abl_in.num_z_bonds = ((const int *) A.in_cols[4])[abl_i];
    abl_in.num_stem_bonds = ((const int *) A.in_cols[5])[abl_i];
    abl_in.cycle = ((const int *) A.in_cols[6])[abl_i];
    abl_in.diff_noise_factor = ((const double *) A.in_cols[7])[abl_i];
    abl_in.dead_ticks = ((const int *) A.in_cols[8])[abl_i];
    abl_in.contact_inhibited_ticks = ((const int *) A.in_cols[9])[abl_i];
    abl_in.motility = ((const double *) A.in_cols[10])[abl_i];
    abl_in.dir = ((const double *) A.in_cols[11])[abl_i];
    abl_in.movement = ((const double *) A.in_cols[12])[abl_i];
    abl_out.type = abl_in.type;
    abl_out.pos = abl_in.pos;
    abl_out.force = abl_in.force;
    abl_out.num_xy_bonds = abl_in.num_xy_bonds;
    abl_out.num_z_bonds = abl_in.num_z_bonds;
    abl_out.num_stem_bonds = abl_in.num_stem_bonds;
    abl_out.cycle = abl_in.cycle;
    abl_out.diff_noise_factor = abl_in.diff_noise_factor;
    abl_out.dead_ticks = abl_in.dead_ticks;
    abl_out.contact_inhibited_ticks = abl_in.contact_inhibited_ticks;
    abl_out.motility = abl_in.motility;
    abl_out.dir = abl_in.dir;
    abl_out.movement = abl_in.movement;
    differentiate(abl_Gr, A.views[abl_r], abl_K, &abl_in, &abl_out);
    ((int *) A.out_cols[0])[abl_i] = abl_out.type;
    ((float3 *) A.out_cols[1])[abl_i] = abl_out.pos;
    ((float3 *) A.out_cols[2])[abl_i] = abl_out.force;
    ((int *) A.out_cols[3])[abl_i] = abl_out.num_xy_bonds;
    ((int *) A.out_cols[4])[abl_i] = abl_out.num_z_bonds;
    ((int *) A.out_cols[5])[abl_i] = abl_out.num_stem_bonds;
    ((int *) A.out_cols[6])[abl_i] = abl_out.cycle;
    ((double *) A.out_cols[7])[abl_i] = abl_out.diff_noise_factor;
    ((int *) A.out_cols[8])[abl_i] = abl_out.dead_ticks;
    ((int *) A.out_cols[9])[abl_i] = abl_out.contact_inhibited_ticks;
    ((double *) A.out_cols[10])[abl_i] = abl_out.motility;
    ((double *) A.out_cols[11])[abl_i] = abl_out.dir;
    ((double *) A.out_cols[12])[abl_i] = abl_out.movement;
}
#ifndef ABL_PERSIST
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ens_differentiate(const __grid_constant__ abl_ens_launch A) {
    abl_ens_body_differentiate(A, blockIdx.x, A.timestep);
}
static int abl_launch_ens_differentiate(const abl_ens_launch *L, cudaStream_t abl_stream) {
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (L->n + abl_block - 1) / abl_block;
    abl_kernel_ens_differentiate<<<abl_grid, abl_block, L->smem, abl_stream>>>(*L);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
#ifndef ABL_PERSIST
static double abl_radius_differentiate(const void *abl_gp) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    return (double) (((double) (125.0)));
}
#endif

__device__ static void death_signal(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Keratinocyte* in, Keratinocyte* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    int num_corn_neighbors = 0;
    if ((in->type == abl_G.K_TYPE_CORN)) {
        return;
    }
    {
        const abl::near_query<3> abl_q2(abl_NB, (double) in->pos.x, (double) in->pos.y, (double) in->pos.z, abl_K.self);
        abl::near_cursor<3> abl_c2(abl_NB, abl_q2);
        auto abl_exact2 = [&](int abl_s) -> bool {
            const float3 abl_p = ((const float3 *) abl_NB.cols[1])[abl_s];
            return !(dist_float3(abl_p, in->pos) > (abl_G.K_WIDTH + abl_G.FORCE_IRADIUS));
        };
        while (abl_c2.fill(abl_q2, abl_exact2)) {
            int abl_pslot2 = abl_c2.slot(0);
            Keratinocyte abl_pnx2;
            abl_pnx2.type = ((const int *) abl_NB.cols[0])[abl_pslot2];
            for (int abl_k = 0; abl_k < abl_c2.cnt; ++abl_k) {
                const int abl_slot2 = abl_pslot2;
                Keratinocyte abl_nx2 = abl_pnx2;
                if (abl_k + 1 < abl_c2.cnt) {
                    abl_pslot2 = abl_c2.slot(abl_k + 1);
                    abl_pnx2.type = ((const int *) abl_NB.cols[0])[abl_pslot2];
                }
                Keratinocyte* other = &abl_nx2;
                {
                    if ((other->type == abl_G.K_TYPE_CORN)) {
                        num_corn_neighbors += 1;
                    }
                }
            }
        }
    }
    double prob = ((float) (num_corn_neighbors * num_corn_neighbors) * 0.01);
    if ((random_3(abl_G, abl_R, 1.0) < prob)) {
        if ((random_3(abl_G, abl_R, 1.0) < 0.01)) {
            out->type = abl_G.K_TYPE_CORN;
        }
    }
}

#ifndef ABL_PERSIST
struct abl_kargs_death_signal {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Keratinocyte in, out;
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
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_death_signal(const __grid_constant__ abl_kargs_death_signal A) {
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
    Keratinocyte abl_in, abl_out;
    abl_in.type = A.in.type[abl_i];
    abl_in.pos = A.in.pos[abl_i];
    abl_in.force = A.in.force[abl_i];
    abl_in.num_xy_bonds = A.in.num_xy_bonds[abl_i];
    abl_in.num_z_bonds = A.in.num_z_bonds[abl_i];
    abl_in.num_stem_bonds = A.in.num_stem_bonds[abl_i];
    abl_in.cycle = A.in.cycle[abl_i];
    abl_in.diff_noise_factor = A.in.diff_noise_factor[abl_i];
    abl_in.dead_ticks = A.in.dead_ticks[abl_i];
    abl_in.contact_inhibited_ticks = A.in.contact_inhibited_ticks[abl_i];
    abl_in.motility = A.in.motility[abl_i];
    abl_in.dir = A.in.dir[abl_i];
    abl_in.movement = A.in.movement[abl_i];
    abl_out = abl_in;
    death_signal(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.type[abl_i] = abl_out.type;
    A.out.pos[abl_i] = abl_out.pos;
    A.out.force[abl_i] = abl_out.force;
    A.out.num_xy_bonds[abl_i] = abl_out.num_xy_bonds;
    A.out.num_z_bonds[abl_i] = abl_out.num_z_bonds;
    A.out.num_stem_bonds[abl_i] = abl_out.num_stem_bonds;
    A.out.cycle[abl_i] = abl_out.cycle;
    A.out.diff_noise_factor[abl_i] = abl_out.diff_noise_factor;
    A.out.dead_ticks[abl_i] = abl_out.dead_ticks;
    A.out.contact_inhibited_ticks[abl_i] = abl_out.contact_inhibited_ticks;
    A.out.motility[abl_i] = abl_out.motility;
    A.out.dir[abl_i] = abl_out.dir;
    A.out.movement[abl_i] = abl_out.movement;
}
static int abl_launch_death_signal(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_death_signal A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.type = (int *) L->in_cols[0];
    A.out.type = (int *) L->out_cols[0];
    A.in.pos = (float3 *) L->in_cols[1];
    A.out.pos = (float3 *) L->out_cols[1];
    A.in.force = (float3 *) L->in_cols[2];
    A.out.force = (float3 *) L->out_cols[2];
    A.in.num_xy_bonds = (int *) L->in_cols[3];
    A.out.num_xy_bonds = (int *) L->out_cols[3];
    A.in.num_z_bonds = (int *) L->in_cols[4];
    A.out.num_z_bonds = (int *) L->out_cols[4];
    A.in.num_stem_bonds = (int *) L->in_cols[5];
    A.out.num_stem_bonds = (int *) L->out_cols[5];
    A.in.cycle = (int *) L->in_cols[6];
    A.out.cycle = (int *) L->out_cols[6];
    A.in.diff_noise_factor = (double *) L->in_cols[7];
    A.out.diff_noise_factor = (double *) L->out_cols[7];
    A.in.dead_ticks = (int *) L->in_cols[8];
    A.out.dead_ticks = (int *) L->out_cols[8];
    A.in.contact_inhibited_ticks = (int *) L->in_cols[9];
    A.out.contact_inhibited_ticks = (int *) L->out_cols[9];
    A.in.motility = (double *) L->in_cols[10];
    A.out.motility = (double *) L->out_cols[10];
    A.in.dir = (double *) L->in_cols[11];
    A.out.dir = (double *) L->out_cols[11];
    A.in.movement = (double *) L->in_cols[12];
    A.out.movement = (double *) L->out_cols[12];
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
    abl_kernel_death_signal<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
__device__ __forceinline__ void abl_ens_body_death_signal(const abl_ens_launch &A, long abl_vb, long abl_ts) {
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
    Keratinocyte abl_in, abl_out;
    abl_in.type = ((const int *) A.in_cols[0])[abl_i];
    abl_in.pos = ((const float3 *) A.in_cols[1])[abl_i];
    abl_in.force = ((const float3 *) A.in_cols[2])[abl_i];
    abl_in.num_xy_bonds = ((const int *) A.in_cols[3])[abl_i];
    abl_in.num_z_bonds = ((const int *) A.in_cols[4])[abl_i];
    abl_in.num_stem_bonds = ((const int *) A.in_cols[5])[abl_i];
    abl_in.cycle = ((const int *) A.in_cols[6])[abl_i];
    abl_in.diff_noise_factor = ((const double *) A.in_cols[7])[abl_i];
    abl_in.dead_ticks = ((const int *) A.in_cols[8])[abl_i];
    abl_in.contact_inhibited_ticks = ((const int *) A.in_cols[9])[abl_i];
    abl_in.motility = ((const double *) A.in_cols[10])[abl_i];
    abl_in.dir = ((const double *) A.in_cols[11])[abl_i];
    abl_in.movement = ((const double *) A.in_cols[12])[abl_i];
    abl_out.type = abl_in.type;
    abl_out.pos = abl_in.pos;
    abl_out.force = abl_in.force;
    abl_out.num_xy_bonds = abl_in.num_xy_bonds;
    abl_out.num_z_bonds = abl_in.num_z_bonds;
    abl_out.num_stem_bonds = abl_in.num_stem_bonds;
    abl_out.cycle = abl_in.cycle;
    abl_out.diff_noise_factor = abl_in.diff_noise_factor;
    abl_out.dead_ticks = abl_in.dead_ticks;
    abl_out.contact_inhibited_ticks = abl_in.contact_inhibited_ticks;
    abl_out.motility = abl_in.motility;
    abl_out.dir = abl_in.dir;
    abl_out.movement = abl_in.movement;
    death_signal(abl_Gr, A.views[abl_r], abl_K, &abl_in, &abl_out);
    ((int *) A.out_cols[0])[abl_i] = abl_out.type;
    ((float3 *) A.out_cols[1])[abl_i] = abl_out.pos;
    ((float3 *) A.out_cols[2])[abl_i] = abl_out.force;
    ((int *) A.out_cols[3])[abl_i] = abl_out.num_xy_bonds;
    ((int *) A.out_cols[4])[abl_i] = abl_out.num_z_bonds;
    ((int *) A.out_cols[5])[abl_i] = abl_out.num_stem_bonds;
    ((int *) A.out_cols[6])[abl_i] = abl_out.cycle;
    ((double *) A.out_cols[7])[abl_i] = abl_out.diff_noise_factor;
    ((int *) A.out_cols[8])[abl_i] = abl_out.dead_ticks;
    ((int *) A.out_cols[9])[abl_i] = abl_out.contact_inhibited_ticks;
    ((double *) A.out_cols[10])[abl_i] = abl_out.motility;
    ((double *) A.out_cols[11])[abl_i] = abl_out.dir;
    ((double *) A.out_cols[12])[abl_i] = abl_out.movement;
}
#ifndef ABL_PERSIST
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ens_death_signal(const __grid_constant__ abl_ens_launch A) {
    abl_ens_body_death_signal(A, blockIdx.x, A.timestep);
}
static int abl_launch_ens_death_signal(const abl_ens_launch *L, cudaStream_t abl_stream) {
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (L->n + abl_block - 1) / abl_block;
    abl_kernel_ens_death_signal<<<abl_grid, abl_block, L->smem, abl_stream>>>(*L);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
#ifndef ABL_PERSIST
static double abl_radius_death_signal(const void *abl_gp) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    return (double) ((abl_G.K_WIDTH + abl_G.FORCE_IRADIUS));
}
#endif

__device__ static void migrate(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Keratinocyte* in, Keratinocyte* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    double x1 = in->pos.x;
    double y1 = in->pos.y;
    double dir1 = in->dir;
    if ((random_3(abl_G, abl_R, 1.0) < 0.1)) {
        dir1 += random_3(abl_G, abl_R, (abl_G.PI / 4.0));
    }
    x1 += (in->motility * cos(dir1));
    y1 += (in->motility * sin(dir1));
    {
        const abl::near_query<3> abl_q3(abl_NB, (double) in->pos.x, (double) in->pos.y, (double) in->pos.z, abl_K.self);
        abl::near_list_cursor<3> abl_c3(abl_NB, abl_q3, abl_K);
        auto abl_exact3 = [&](int abl_s) -> bool {
            const float3 abl_p = ((const float3 *) abl_NB.cols[1])[abl_s];
            return !(dist_float3(abl_p, in->pos) > abl_G.K_WIDTH);
        };
        while (abl_c3.fill(abl_q3, abl_exact3)) {
            int abl_pslot3 = abl_c3.slot(0);
            Keratinocyte abl_pnx3;
            abl_pnx3.pos = ((const float3 *) abl_NB.cols[1])[abl_pslot3];
            abl_pnx3.motility = ((const double *) abl_NB.cols[10])[abl_pslot3];
            unsigned long long abl_dm3_0 = 0ull;
            for (int abl_k = 0; abl_k < abl_c3.cnt; ++abl_k) {
                const int abl_slot3 = abl_pslot3;
                Keratinocyte abl_nx3 = abl_pnx3;
                if (abl_k + 1 < abl_c3.cnt) {
                    abl_pslot3 = abl_c3.slot(abl_k + 1);
                    abl_pnx3.pos = ((const float3 *) abl_NB.cols[1])[abl_pslot3];
                    abl_pnx3.motility = ((const double *) abl_NB.cols[10])[abl_pslot3];
                }
                Keratinocyte* other = &abl_nx3;
                {
                    if (((in->type != abl_G.K_TYPE_TA) && (in->type != abl_G.K_TYPE_HACAT))) {
                        continue;
                    }
                    if ((on_substrate_surface(abl_G, abl_R, other->pos.z) && (other->motility == 0))) abl_dm3_0 |= 1ull << abl_k;
                }
            }
            for (unsigned long long abl_m = abl_dm3_0; abl_m; abl_m &= abl_m - 1ull) {
                const int abl_slot3 = abl_c3.slot(__ffsll((long long) abl_m) - 1);
                Keratinocyte abl_nx3;
                abl_nx3.pos = ((const float3 *) abl_NB.cols[1])[abl_slot3];
                abl_nx3.motility = ((const double *) abl_NB.cols[10])[abl_slot3];
                Keratinocyte* other = &abl_nx3;
                {
                    dir1 -= abl_G.PI;
                    if ((dir1 > (2.0 * abl_G.PI))) {
                        dir1 -= (2.0 * abl_G.PI);
                    }
                    x1 = (in->pos.x + (in->motility * cos(dir1)));
                    y1 = (in->pos.y + (in->motility * sin(dir1)));
                }
            }
        }
    }
    if ((x1 > abl_G.SURFACE_WIDTH)) {
        x1 = (abl_G.SURFACE_WIDTH - (in->motility * random_3(abl_G, abl_R, 1.0)));
        dir1 = (abl_G.PI + ((abl_G.PI * abl_random(abl_R, (-0.5), 0.5)) / 4.0));
    }
    if ((x1 < 0)) {
        x1 = (in->motility * random_3(abl_G, abl_R, 1.0));
        dir1 = ((abl_G.PI * abl_random(abl_R, (-0.5), 0.5)) / 4.0);
    }
    if ((y1 > abl_G.SURFACE_WIDTH)) {
        y1 = (abl_G.SURFACE_WIDTH - (in->motility * random_3(abl_G, abl_R, 1.0)));
        dir1 = (((3.0 * abl_G.PI) / 2.0) + ((abl_G.PI * abl_random(abl_R, (-0.5), 0.5)) / 4.0));
    }
    if ((y1 < 0)) {
        y1 = (in->motility * random_3(abl_G, abl_R, 1.0));
        dir1 = (((abl_G.PI / 2.0) * abl_random(abl_R, (-0.5), 0.5)) / 4.0);
    }
    out->pos.x = x1;
    out->pos.y = y1;
    out->dir = dir1;
}

#ifndef ABL_PERSIST
struct abl_kargs_migrate {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Keratinocyte in, out;
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
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_migrate(const __grid_constant__ abl_kargs_migrate A) {
    int abl_j;
    {
        const abl_globals &abl_G = A.G;
        const long abl_t1 = (long) blockIdx.x * blockDim.x + threadIdx.x;
        const bool abl_has = abl_t1 < A.n;
        const long abl_i1 = abl_has ? (A.visit ? (long) A.visit[abl_t1] : abl_t1) : 0;
        const float3 abl_p1 = abl_has ? A.in.pos[abl_i1] : float3{};
        const abl::near_query<3> abl_q0(A.NB, (double) abl_p1.x, (double) abl_p1.y, (double) abl_p1.z, abl_has ? abl_i1 : -1);
        auto abl_x0 = [&](int abl_s) -> bool {
            const float3 abl_p = ((const float3 *) A.NB.cols[1])[abl_s];
            return !(dist_float3(abl_p, abl_p1) > abl_G.K_WIDTH);
        };
        abl_j = abl::presort_block<3>(A.NB, abl_has, abl_q0, abl_x0);
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
    Keratinocyte abl_in, abl_out;
    abl_in.type = A.in.type[abl_i];
    abl_in.pos = A.in.pos[abl_i];
    abl_in.force = A.in.force[abl_i];
    abl_in.num_xy_bonds = A.in.num_xy_bonds[abl_i];
    abl_in.num_z_bonds = A.in.num_z_bonds[abl_i];
    abl_in.num_stem_bonds = A.in.num_stem_bonds[abl_i];
    abl_in.cycle = A.in.cycle[abl_i];
    abl_in.diff_noise_factor = A.in.diff_noise_factor[abl_i];
    abl_in.dead_ticks = A.in.dead_ticks[abl_i];
    abl_in.contact_inhibited_ticks = A.in.contact_inhibited_ticks[abl_i];
    abl_in.motility = A.in.motility[abl_i];
    abl_in.dir = A.in.dir[abl_i];
    abl_in.movement = A.in.movement[abl_i];
    abl_out = abl_in;
    migrate(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.type[abl_i] = abl_out.type;
    A.out.pos[abl_i] = abl_out.pos;
    A.out.force[abl_i] = abl_out.force;
    A.out.num_xy_bonds[abl_i] = abl_out.num_xy_bonds;
    A.out.num_z_bonds[abl_i] = abl_out.num_z_bonds;
    A.out.num_stem_bonds[abl_i] = abl_out.num_stem_bonds;
    A.out.cycle[abl_i] = abl_out.cycle;
    A.out.diff_noise_factor[abl_i] = abl_out.diff_noise_factor;
    A.out.dead_ticks[abl_i] = abl_out.dead_ticks;
    A.out.contact_inhibited_ticks[abl_i] = abl_out.contact_inhibited_ticks;
    A.out.motility[abl_i] = abl_out.motility;
    A.out.dir[abl_i] = abl_out.dir;
    A.out.movement[abl_i] = abl_out.movement;
}
static int abl_launch_migrate(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_migrate A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.type = (int *) L->in_cols[0];
    A.out.type = (int *) L->out_cols[0];
    A.in.pos = (float3 *) L->in_cols[1];
    A.out.pos = (float3 *) L->out_cols[1];
    A.in.force = (float3 *) L->in_cols[2];
    A.out.force = (float3 *) L->out_cols[2];
    A.in.num_xy_bonds = (int *) L->in_cols[3];
    A.out.num_xy_bonds = (int *) L->out_cols[3];
    A.in.num_z_bonds = (int *) L->in_cols[4];
    A.out.num_z_bonds = (int *) L->out_cols[4];
    A.in.num_stem_bonds = (int *) L->in_cols[5];
    A.out.num_stem_bonds = (int *) L->out_cols[5];
    A.in.cycle = (int *) L->in_cols[6];
    A.out.cycle = (int *) L->out_cols[6];
    A.in.diff_noise_factor = (double *) L->in_cols[7];
    A.out.diff_noise_factor = (double *) L->out_cols[7];
    A.in.dead_ticks = (int *) L->in_cols[8];
    A.out.dead_ticks = (int *) L->out_cols[8];
    A.in.contact_inhibited_ticks = (int *) L->in_cols[9];
    A.out.contact_inhibited_ticks = (int *) L->out_cols[9];
    A.in.motility = (double *) L->in_cols[10];
    A.out.motility = (double *) L->out_cols[10];
    A.in.dir = (double *) L->in_cols[11];
    A.out.dir = (double *) L->out_cols[11];
    A.in.movement = (double *) L->in_cols[12];
    A.out.movement = (double *) L->out_cols[12];
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
    abl_kernel_migrate<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
__device__ __forceinline__ void abl_ens_body_migrate(const abl_ens_launch &A, long abl_vb, long abl_ts) {
    int abl_j;
    {
        const long abl_t1 = abl_vb * blockDim.x + threadIdx.x;
        const bool abl_has = abl_t1 < A.n;
        const long abl_i1 = abl_has ? (A.visit_order ? (long) A.visit_order[abl_t1] : abl_t1) : 0;
        const int abl_r1 = abl_has ? A.replica[abl_i1] : 0;
        const abl_globals &abl_G = ((const abl_globals *) A.globals)[abl_r1];
        const abl_near_view &abl_V1 = A.views[abl_r1];
        const float3 abl_p1 = abl_has ? ((const float3 *) A.in_cols[1])[abl_i1] : float3{};
        const abl::near_query<3> abl_q0(abl_V1, (double) abl_p1.x, (double) abl_p1.y, (double) abl_p1.z, abl_has ? abl_i1 : -1);
        auto abl_x0 = [&](int abl_s) -> bool {
            const float3 abl_p = ((const float3 *) abl_V1.cols[1])[abl_s];
            return !(dist_float3(abl_p, abl_p1) > abl_G.K_WIDTH);
        };
        abl_j = abl::presort_block<3>(abl_V1, abl_has, abl_q0, abl_x0);
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
    Keratinocyte abl_in, abl_out;
    abl_in.type = ((const int *) A.in_cols[0])[abl_i];
    abl_in.pos = ((const float3 *) A.in_cols[1])[abl_i];
    abl_in.force = ((const float3 *) A.in_cols[2])[abl_i];
    abl_in.num_xy_bonds = ((const int *) A.in_cols[3])[abl_i];
    abl_in.num_z_bonds = ((const int *) A.in_cols[4])[abl_i];
    abl_in.num_stem_bonds = ((const int *) A.in_cols[5])[abl_i];
    abl_in.cycle = ((const int *) A.in_cols[6])[abl_i];
    abl_in.diff_noise_factor = ((const double *) A.in_cols[7])[abl_i];
    abl_in.dead_ticks = ((const int *) A.in_cols[8])[abl_i];
    abl_in.contact_inhibited_ticks = ((const int *) A.in_cols[9])[abl_i];
    abl_in.motility = ((const double *) A.in_cols[10])[abl_i];
    abl_in.dir = ((const double *) A.in_cols[11])[abl_i];
    abl_in.movement = ((const double *) A.in_cols[12])[abl_i];
    abl_out.type = abl_in.type;
    abl_out.pos = abl_in.pos;
    abl_out.force = abl_in.force;
    abl_out.num_xy_bonds = abl_in.num_xy_bonds;
    abl_out.num_z_bonds = abl_in.num_z_bonds;
    abl_out.num_stem_bonds = abl_in.num_stem_bonds;
    abl_out.cycle = abl_in.cycle;
    abl_out.diff_noise_factor = abl_in.diff_noise_factor;
    abl_out.dead_ticks = abl_in.dead_ticks;
    abl_out.contact_inhibited_ticks = abl_in.contact_inhibited_ticks;
    abl_out.motility = abl_in.motility;
    abl_out.dir = abl_in.dir;
    abl_out.movement = abl_in.movement;
    migrate(abl_Gr, A.views[abl_r], abl_K, &abl_in, &abl_out);
    ((int *) A.out_cols[0])[abl_i] = abl_out.type;
    ((float3 *) A.out_cols[1])[abl_i] = abl_out.pos;
    ((float3 *) A.out_cols[2])[abl_i] = abl_out.force;
    ((int *) A.out_cols[3])[abl_i] = abl_out.num_xy_bonds;
    ((int *) A.out_cols[4])[abl_i] = abl_out.num_z_bonds;
    ((int *) A.out_cols[5])[abl_i] = abl_out.num_stem_bonds;
    ((int *) A.out_cols[6])[abl_i] = abl_out.cycle;
    ((double *) A.out_cols[7])[abl_i] = abl_out.diff_noise_factor;
    ((int *) A.out_cols[8])[abl_i] = abl_out.dead_ticks;
    ((int *) A.out_cols[9])[abl_i] = abl_out.contact_inhibited_ticks;
    ((double *) A.out_cols[10])[abl_i] = abl_out.motility;
    ((double *) A.out_cols[11])[abl_i] = abl_out.dir;
    ((double *) A.out_cols[12])[abl_i] = abl_out.movement;
}
#ifndef ABL_PERSIST
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ens_migrate(const __grid_constant__ abl_ens_launch A) {
    abl_ens_body_migrate(A, blockIdx.x, A.timestep);
}
static int abl_launch_ens_migrate(const abl_ens_launch *L, cudaStream_t abl_stream) {
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (L->n + abl_block - 1) / abl_block;
    abl_kernel_ens_migrate<<<abl_grid, abl_block, L->smem, abl_stream>>>(*L);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
#ifndef ABL_PERSIST
static double abl_radius_migrate(const void *abl_gp) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    return (double) (abl_G.K_WIDTH);
}
#endif

__device__ static void resolve_forces(const abl_globals &abl_G, const abl_near_view &abl_NB, abl::step_ctx &abl_K, Keratinocyte* in, Keratinocyte* out) {
    abl::rng &abl_R = abl_K.R;
    (void) abl_R; (void) abl_NB;
    float3 new_force = in->force;
    int num_xy_bonds = 0;
    int num_z_bonds = 0;
    int num_stem_bonds = 0;
    {
        const abl::near_query<3> abl_q4(abl_NB, (double) in->pos.x, (double) in->pos.y, (double) in->pos.z, abl_K.self);
        abl::near_list_cursor<3> abl_c4(abl_NB, abl_q4, abl_K);
        auto abl_exact4 = [&](int abl_s) -> bool {
            const float3 abl_p = ((const float3 *) abl_NB.cols[1])[abl_s];
            return !(dist_float3(abl_p, in->pos) > (abl_G.K_WIDTH + abl_G.FORCE_IRADIUS));
        };
        while (abl_c4.fill(abl_q4, abl_exact4)) {
            int abl_pslot4 = abl_c4.slot(0);
            Keratinocyte abl_pnx4;
            abl_pnx4.type = ((const int *) abl_NB.cols[0])[abl_pslot4];
            abl_pnx4.pos = ((const float3 *) abl_NB.cols[1])[abl_pslot4];
            for (int abl_k = 0; abl_k < abl_c4.cnt; ++abl_k) {
                const int abl_slot4 = abl_pslot4;
                Keratinocyte abl_nx4 = abl_pnx4;
                if (abl_k + 1 < abl_c4.cnt) {
                    abl_pslot4 = abl_c4.slot(abl_k + 1);
                    abl_pnx4.type = ((const int *) abl_NB.cols[0])[abl_pslot4];
                    abl_pnx4.pos = ((const float3 *) abl_NB.cols[1])[abl_pslot4];
                }
                Keratinocyte* other = &abl_nx4;
                {
                    double distance = dist_float3(in->pos, other->pos);
                    if ((distance == 0.0)) continue;
                    double separation_distance = (distance - abl_G.K_WIDTH);
                    if ((other->pos.z >= in->pos.z)) {
                        if (((other->pos.z - in->pos.z) > (abl_G.K_WIDTH / 2.0))) {
                            num_z_bonds += 1;
                        } else {
                            num_xy_bonds += 1;
                        }
                    }
                    if ((other->type == abl_G.K_TYPE_STEM)) {
                        num_stem_bonds += 1;
                    }
                    double force = ((separation_distance > 0) ? abl_G.FORCE_MATRIX[(in->type + (5 * other->type))] : abl_G.FORCE_REP);
                    if (on_substrate_surface(abl_G, abl_R, in->pos.z)) {
                        force *= abl_G.DOWNWARD_FORCE[in->type];
                    }
                    force *= abl_G.FORCE_DAMPENER;
                    new_force = float3_add(new_force, float3_div_scalar(float3_mul_scalar(float3_mul_scalar(float3_sub(other->pos, in->pos), force), separation_distance), distance));
                }
            }
        }
    }
    if ((in->pos.z <= (abl_G.K_WIDTH * 1.5))) {
        new_force.z -= abl_G.SUBSTRATE_FORCE[in->type];
    }
    out->num_xy_bonds = num_xy_bonds;
    out->num_z_bonds = num_z_bonds;
    out->num_stem_bonds = num_stem_bonds;
    float3 new_pos = float3_add(in->pos, new_force);
    if ((new_pos.x < 0)) {
        new_pos.x = 0;
    }
    if ((new_pos.y < 0)) {
        new_pos.y = 0;
    }
    if ((new_pos.z < 0)) {
        new_pos.z = 0;
    }
    if ((new_pos.x > abl_G.SURFACE_WIDTH)) {
        new_pos.x = abl_G.SURFACE_WIDTH;
    }
    if ((new_pos.y > abl_G.SURFACE_WIDTH)) {
        new_pos.y = abl_G.SURFACE_WIDTH;
    }
    out->movement = length_float3(float3_sub(new_pos, in->pos));
    out->pos = new_pos;
}

#ifndef ABL_PERSIST
struct abl_kargs_resolve_forces {
    abl_globals G;
    long n;
    const int *visit;
    abl_cols_Keratinocyte in, out;
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
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_resolve_forces(const __grid_constant__ abl_kargs_resolve_forces A) {
    int abl_j;
    {
        const abl_globals &abl_G = A.G;
        const long abl_t1 = (long) blockIdx.x * blockDim.x + threadIdx.x;
        const bool abl_has = abl_t1 < A.n;
        const long abl_i1 = abl_has ? (A.visit ? (long) A.visit[abl_t1] : abl_t1) : 0;
        const float3 abl_p1 = abl_has ? A.in.pos[abl_i1] : float3{};
        const abl::near_query<3> abl_q0(A.NB, (double) abl_p1.x, (double) abl_p1.y, (double) abl_p1.z, abl_has ? abl_i1 : -1);
        auto abl_x0 = [&](int abl_s) -> bool {
            const float3 abl_p = ((const float3 *) A.NB.cols[1])[abl_s];
            return !(dist_float3(abl_p, abl_p1) > (abl_G.K_WIDTH + abl_G.FORCE_IRADIUS));
        };
        abl_j = abl::presort_block<3>(A.NB, abl_has, abl_q0, abl_x0);
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
    Keratinocyte abl_in, abl_out;
    abl_in.type = A.in.type[abl_i];
    abl_in.pos = A.in.pos[abl_i];
    abl_in.force = A.in.force[abl_i];
    abl_in.num_xy_bonds = A.in.num_xy_bonds[abl_i];
    abl_in.num_z_bonds = A.in.num_z_bonds[abl_i];
    abl_in.num_stem_bonds = A.in.num_stem_bonds[abl_i];
    abl_in.cycle = A.in.cycle[abl_i];
    abl_in.diff_noise_factor = A.in.diff_noise_factor[abl_i];
    abl_in.dead_ticks = A.in.dead_ticks[abl_i];
    abl_in.contact_inhibited_ticks = A.in.contact_inhibited_ticks[abl_i];
    abl_in.motility = A.in.motility[abl_i];
    abl_in.dir = A.in.dir[abl_i];
    abl_in.movement = A.in.movement[abl_i];
    abl_out = abl_in;
    resolve_forces(A.G, A.NB, abl_K, &abl_in, &abl_out);
    A.out.type[abl_i] = abl_out.type;
    A.out.pos[abl_i] = abl_out.pos;
    A.out.force[abl_i] = abl_out.force;
    A.out.num_xy_bonds[abl_i] = abl_out.num_xy_bonds;
    A.out.num_z_bonds[abl_i] = abl_out.num_z_bonds;
    A.out.num_stem_bonds[abl_i] = abl_out.num_stem_bonds;
    A.out.cycle[abl_i] = abl_out.cycle;
    A.out.diff_noise_factor[abl_i] = abl_out.diff_noise_factor;
    A.out.dead_ticks[abl_i] = abl_out.dead_ticks;
    A.out.contact_inhibited_ticks[abl_i] = abl_out.contact_inhibited_ticks;
    A.out.motility[abl_i] = abl_out.motility;
    A.out.dir[abl_i] = abl_out.dir;
    A.out.movement[abl_i] = abl_out.movement;
}
static int abl_launch_resolve_forces(const abl_step_launch *L, cudaStream_t abl_stream) {
    abl_kargs_resolve_forces A;
    A.G = *(const abl_globals *) L->globals;
    A.n = L->n;
    A.visit = L->visit_order;
    A.in.type = (int *) L->in_cols[0];
    A.out.type = (int *) L->out_cols[0];
    A.in.pos = (float3 *) L->in_cols[1];
    A.out.pos = (float3 *) L->out_cols[1];
    A.in.force = (float3 *) L->in_cols[2];
    A.out.force = (float3 *) L->out_cols[2];
    A.in.num_xy_bonds = (int *) L->in_cols[3];
    A.out.num_xy_bonds = (int *) L->out_cols[3];
    A.in.num_z_bonds = (int *) L->in_cols[4];
    A.out.num_z_bonds = (int *) L->out_cols[4];
    A.in.num_stem_bonds = (int *) L->in_cols[5];
    A.out.num_stem_bonds = (int *) L->out_cols[5];
    A.in.cycle = (int *) L->in_cols[6];
    A.out.cycle = (int *) L->out_cols[6];
    A.in.diff_noise_factor = (double *) L->in_cols[7];
    A.out.diff_noise_factor = (double *) L->out_cols[7];
    A.in.dead_ticks = (int *) L->in_cols[8];
    A.out.dead_ticks = (int *) L->out_cols[8];
    A.in.contact_inhibited_ticks = (int *) L->in_cols[9];
    A.out.contact_inhibited_ticks = (int *) L->out_cols[9];
    A.in.motility = (double *) L->in_cols[10];
    A.out.motility = (double *) L->out_cols[10];
    A.in.dir = (double *) L->in_cols[11];
    A.out.dir = (double *) L->out_cols[11];
    A.in.movement = (double *) L->in_cols[12];
    A.out.movement = (double *) L->out_cols[12];
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
    abl_kernel_resolve_forces<<<abl_grid, abl_block, L->smem, abl_stream>>>(A);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
__device__ __forceinline__ void abl_ens_body_resolve_forces(const abl_ens_launch &A, long abl_vb, long abl_ts) {
    int abl_j;
    {
        const long abl_t1 = abl_vb * blockDim.x + threadIdx.x;
        const bool abl_has = abl_t1 < A.n;
        const long abl_i1 = abl_has ? (A.visit_order ? (long) A.visit_order[abl_t1] : abl_t1) : 0;
        const int abl_r1 = abl_has ? A.replica[abl_i1] : 0;
        const abl_globals &abl_G = ((const abl_globals *) A.globals)[abl_r1];
        const abl_near_view &abl_V1 = A.views[abl_r1];
        const float3 abl_p1 = abl_has ? ((const float3 *) A.in_cols[1])[abl_i1] : float3{};
        const abl::near_query<3> abl_q0(abl_V1, (double) abl_p1.x, (double) abl_p1.y, (double) abl_p1.z, abl_has ? abl_i1 : -1);
        auto abl_x0 = [&](int abl_s) -> bool {
            const float3 abl_p = ((const float3 *) abl_V1.cols[1])[abl_s];
            return !(dist_float3(abl_p, abl_p1) > (abl_G.K_WIDTH + abl_G.FORCE_IRADIUS));
        };
        abl_j = abl::presort_block<3>(abl_V1, abl_has, abl_q0, abl_x0);
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
    Keratinocyte abl_in, abl_out;
    abl_in.type = ((const int *) A.in_cols[0])[abl_i];
    abl_in.pos = ((const float3 *) A.in_cols[1])[abl_i];
    abl_in.force = ((const float3 *) A.in_cols[2])[abl_i];
    abl_in.num_xy_bonds = ((const int *) A.in_cols[3])[abl_i];
    abl_in.num_z_bonds = ((const int *) A.in_cols[4])[abl_i];
    abl_in.num_stem_bonds = ((const int *) A.in_cols[5])[abl_i];
    abl_in.cycle = ((const int *) A.in_cols[6])[abl_i];
    abl_in.diff_noise_factor = ((const double *) A.in_cols[7])[abl_i];
    abl_in.dead_ticks = ((const int *) A.in_cols[8])[abl_i];
    abl_in.contact_inhibited_ticks = ((const int *) A.in_cols[9])[abl_i];
    abl_in.motility = ((const double *) A.in_cols[10])[abl_i];
    abl_in.dir = ((const double *) A.in_cols[11])[abl_i];
    abl_in.movement = ((const double *) A.in_cols[12])[abl_i];
    abl_out.type = abl_in.type;
    abl_out.pos = abl_in.pos;
    abl_out.force = abl_in.force;
    abl_out.num_xy_bonds = abl_in.num_xy_bonds;
    abl_out.num_z_bonds = abl_in.num_z_bonds;
    abl_out.num_stem_bonds = abl_in.num_stem_bonds;
    abl_out.cycle = abl_in.cycle;
    abl_out.diff_noise_factor = abl_in.diff_noise_factor;
    abl_out.dead_ticks = abl_in.dead_ticks;
    abl_out.contact_inhibited_ticks = abl_in.contact_inhibited_ticks;
    abl_out.motility = abl_in.motility;
    abl_out.dir = abl_in.dir;
    abl_out.movement = abl_in.movement;
    resolve_forces(abl_Gr, A.views[abl_r], abl_K, &abl_in, &abl_out);
    ((int *) A.out_cols[0])[abl_i] = abl_out.type;
    ((float3 *) A.out_cols[1])[abl_i] = abl_out.pos;
    ((float3 *) A.out_cols[2])[abl_i] = abl_out.force;
    ((int *) A.out_cols[3])[abl_i] = abl_out.num_xy_bonds;
    ((int *) A.out_cols[4])[abl_i] = abl_out.num_z_bonds;
    ((int *) A.out_cols[5])[abl_i] = abl_out.num_stem_bonds;
    ((int *) A.out_cols[6])[abl_i] = abl_out.cycle;
    ((double *) A.out_cols[7])[abl_i] = abl_out.diff_noise_factor;
    ((int *) A.out_cols[8])[abl_i] = abl_out.dead_ticks;
    ((int *) A.out_cols[9])[abl_i] = abl_out.contact_inhibited_ticks;
    ((double *) A.out_cols[10])[abl_i] = abl_out.motility;
    ((double *) A.out_cols[11])[abl_i] = abl_out.dir;
    ((double *) A.out_cols[12])[abl_i] = abl_out.movement;
}
#ifndef ABL_PERSIST
__global__ void __launch_bounds__(ABL_STEP_BLOCK, ABL_STEP_MIN_BLOCKS) abl_kernel_ens_resolve_forces(const __grid_constant__ abl_ens_launch A) {
    abl_ens_body_resolve_forces(A, blockIdx.x, A.timestep);
}
static int abl_launch_ens_resolve_forces(const abl_ens_launch *L, cudaStream_t abl_stream) {
    const int abl_block = L->block > 0 && L->block <= ABL_STEP_BLOCK ? L->block : ABL_STEP_BLOCK;
    const long abl_grid = (L->n + abl_block - 1) / abl_block;
    abl_kernel_ens_resolve_forces<<<abl_grid, abl_block, L->smem, abl_stream>>>(*L);
    return cudaGetLastError() == cudaSuccess ? ABL_OK : ABL_E_CUDA;
}
#endif
#ifndef ABL_PERSIST
static double abl_radius_resolve_forces(const void *abl_gp) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    return (double) ((abl_G.K_WIDTH + abl_G.FORCE_IRADIUS));
}
#endif

static int abl_seq_gather_stats(abl_ctx *abl_C, const void *abl_gp) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R_host;
    abl::rng &abl_R = abl_R_host;
    (void) abl_G; (void) abl_R;
    int num_stem = abl_seq_count_eq(abl_C, 0, 0, (int) abl_G.K_TYPE_STEM);
    int num_ta = abl_seq_count_eq(abl_C, 0, 0, (int) abl_G.K_TYPE_TA);
    int num_comm = abl_seq_count_eq(abl_C, 0, 0, (int) abl_G.K_TYPE_COMM);
    int num_corn = abl_seq_count_eq(abl_C, 0, 0, (int) abl_G.K_TYPE_CORN);
    int num_hacat = abl_seq_count_eq(abl_C, 0, 0, (int) abl_G.K_TYPE_HACAT);
    double exec_time = abl_seq_exec_time(abl_C);
    abl_log_csv(abl_C, "%d,%d,%d,%d,%d,%f\n", num_stem, num_ta, num_comm, num_corn, num_hacat, exec_time);
    return ABL_OK;
}

#ifndef ABL_PERSIST
static const abl_member_desc abl_members_Keratinocyte[] = {
    {"type", ABL_T_INT, 1, 4, 0},
    {"pos", ABL_T_FLOAT3, 3, 8, 1},
    {"force", ABL_T_FLOAT3, 3, 8, 0},
    {"num_xy_bonds", ABL_T_INT, 1, 4, 0},
    {"num_z_bonds", ABL_T_INT, 1, 4, 0},
    {"num_stem_bonds", ABL_T_INT, 1, 4, 0},
    {"cycle", ABL_T_INT, 1, 4, 0},
    {"diff_noise_factor", ABL_T_FLOAT, 1, 8, 0},
    {"dead_ticks", ABL_T_INT, 1, 4, 0},
    {"contact_inhibited_ticks", ABL_T_INT, 1, 4, 0},
    {"motility", ABL_T_FLOAT, 1, 8, 0},
    {"dir", ABL_T_FLOAT, 1, 8, 0},
    {"movement", ABL_T_FLOAT, 1, 8, 0},
};
static const abl_agent_desc abl_agents[] = {
    {"Keratinocyte", 13, abl_members_Keratinocyte, 1, 3},
};
static const abl_global_desc abl_global_table[] = {
    {"PI", ABL_T_FLOAT, offsetof(abl_globals, PI)},
    {"K_WIDTH", ABL_T_FLOAT, offsetof(abl_globals, K_WIDTH)},
    {"FORCE_IRADIUS", ABL_T_FLOAT, offsetof(abl_globals, FORCE_IRADIUS)},
    {"BASEMENT_MAX_Z", ABL_T_FLOAT, offsetof(abl_globals, BASEMENT_MAX_Z)},
    {"MAX_TO_G0_CONTACT_INHIBITED_TICKS", ABL_T_INT, offsetof(abl_globals, MAX_TO_G0_CONTACT_INHIBITED_TICKS)},
    {"MAX_DEAD_TICKS", ABL_T_INT, offsetof(abl_globals, MAX_DEAD_TICKS)},
    {"MAX_NUM_LATERAL_BONDS", ABL_T_INT, offsetof(abl_globals, MAX_NUM_LATERAL_BONDS)},
    {"FORCE_REP", ABL_T_FLOAT, offsetof(abl_globals, FORCE_REP)},
    {"FORCE_DAMPENER", ABL_T_FLOAT, offsetof(abl_globals, FORCE_DAMPENER)},
    {"calcium_level", ABL_T_FLOAT, offsetof(abl_globals, calcium_level)},
    {"K_TYPE_STEM", ABL_T_INT, offsetof(abl_globals, K_TYPE_STEM)},
    {"K_TYPE_TA", ABL_T_INT, offsetof(abl_globals, K_TYPE_TA)},
    {"K_TYPE_COMM", ABL_T_INT, offsetof(abl_globals, K_TYPE_COMM)},
    {"K_TYPE_CORN", ABL_T_INT, offsetof(abl_globals, K_TYPE_CORN)},
    {"K_TYPE_HACAT", ABL_T_INT, offsetof(abl_globals, K_TYPE_HACAT)},
    {"num_agents", ABL_T_INT, offsetof(abl_globals, num_agents)},
    {"num_timesteps", ABL_T_INT, offsetof(abl_globals, num_timesteps)},
    {"SURFACE_WIDTH", ABL_T_FLOAT, offsetof(abl_globals, SURFACE_WIDTH)},
    {nullptr, 0, 0}
};
static void abl_env_bounds(const void *abl_gp, double *abl_min, double *abl_max) {
    const abl_globals &abl_G = *(const abl_globals *) abl_gp;
    abl::rng abl_R;
    (void) abl_G; (void) abl_R;
    float3 abl_lo = float3_fill(0);
    float3 abl_hi = float3_create(abl_G.SURFACE_WIDTH, abl_G.SURFACE_WIDTH, 100);
    abl_min[0] = abl_lo.x; abl_min[1] = abl_lo.y; abl_min[2] = abl_lo.z;
    abl_max[0] = abl_hi.x; abl_max[1] = abl_hi.y; abl_max[2] = abl_hi.z;
}
static const abl_step_desc abl_steps[] = {
    {"cycle", 0, -1, 1, nullptr, 0u, 0u, abl_launch_cycle, 0, 0, 1, nullptr, 1, 0, 576u, 0},
    {"differentiate", 0, 0, 1, abl_radius_differentiate, 3u, 0u, abl_launch_differentiate, 0, -1, 1, abl_launch_ens_differentiate, 0, 1, 257u, 1},
    {"death_signal", 0, 0, 0, abl_radius_death_signal, 3u, 0u, abl_launch_death_signal, 0, -1, 1, abl_launch_ens_death_signal, 1, 0, 1u, 1},
    {"migrate", 0, 0, 1, abl_radius_migrate, 1026u, 2048u, abl_launch_migrate, 0, -1, 1, abl_launch_ens_migrate, 1, 1, 2050u, 1},
    {"resolve_forces", 0, 0, 1, abl_radius_resolve_forces, 3u, 4154u, abl_launch_resolve_forces, 0, -1, 1, abl_launch_ens_resolve_forces, 0, 1, 4154u, 1},
};
static const abl_step_desc abl_steps_ordered[] = {
    abl_steps[0],
    abl_steps[1],
    abl_steps[2],
    abl_steps[3],
    abl_steps[4],
    {nullptr, 0, -1, 0, nullptr, 0u, 0u, nullptr, 0, -1, 0, nullptr, 0}
};
extern const abl_model_desc abl_desc = {
    "keratinocyte", 1, abl_agents, 5, abl_steps_ordered, sizeof(abl_globals), &abl_globals_default, 18, abl_global_table, 3, abl_env_bounds, nullptr, 0, abl_seq_gather_stats, nullptr
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
        size_t n = agents.agents_Keratinocyte.len;
        const Keratinocyte *aos = (const Keratinocyte *) agents.agents_Keratinocyte.values;
        int *c0 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c0[i] = aos[i].type;
        float3 *c1 = (float3 *) std::malloc(sizeof(float3) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c1[i] = aos[i].pos;
        float3 *c2 = (float3 *) std::malloc(sizeof(float3) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c2[i] = aos[i].force;
        int *c3 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c3[i] = aos[i].num_xy_bonds;
        int *c4 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c4[i] = aos[i].num_z_bonds;
        int *c5 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c5[i] = aos[i].num_stem_bonds;
        int *c6 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c6[i] = aos[i].cycle;
        double *c7 = (double *) std::malloc(sizeof(double) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c7[i] = aos[i].diff_noise_factor;
        int *c8 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c8[i] = aos[i].dead_ticks;
        int *c9 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c9[i] = aos[i].contact_inhibited_ticks;
        double *c10 = (double *) std::malloc(sizeof(double) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c10[i] = aos[i].motility;
        double *c11 = (double *) std::malloc(sizeof(double) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c11[i] = aos[i].dir;
        double *c12 = (double *) std::malloc(sizeof(double) * (n ? n : 1));
        for (size_t i = 0; i < n; i++) c12[i] = aos[i].movement;
        const void *cols[] = {c0, c1, c2, c3, c4, c5, c6, c7, c8, c9, c10, c11, c12};
        abl_check(abl_upload(ctx, 0, cols, n), "abl_upload");
        std::free(c0);
        std::free(c1);
        std::free(c2);
        std::free(c3);
        std::free(c4);
        std::free(c5);
        std::free(c6);
        std::free(c7);
        std::free(c8);
        std::free(c9);
        std::free(c10);
        std::free(c11);
        std::free(c12);
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
        int *c0 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        float3 *c1 = (float3 *) std::malloc(sizeof(float3) * (n ? n : 1));
        float3 *c2 = (float3 *) std::malloc(sizeof(float3) * (n ? n : 1));
        int *c3 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        int *c4 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        int *c5 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        int *c6 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        double *c7 = (double *) std::malloc(sizeof(double) * (n ? n : 1));
        int *c8 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        int *c9 = (int *) std::malloc(sizeof(int) * (n ? n : 1));
        double *c10 = (double *) std::malloc(sizeof(double) * (n ? n : 1));
        double *c11 = (double *) std::malloc(sizeof(double) * (n ? n : 1));
        double *c12 = (double *) std::malloc(sizeof(double) * (n ? n : 1));
        void *cols[] = {c0, c1, c2, c3, c4, c5, c6, c7, c8, c9, c10, c11, c12};
        size_t cap = n;
        abl_check(abl_download(ctx, 0, cols, &cap), "abl_download");
        dyn_array_clean(&agents.agents_Keratinocyte);
        agents.agents_Keratinocyte = dyn_array_create_fixed(sizeof(Keratinocyte), n);
        Keratinocyte *aos = (Keratinocyte *) agents.agents_Keratinocyte.values;
        for (size_t i = 0; i < n; i++) {
            aos[i].type = c0[i];
            aos[i].pos = c1[i];
            aos[i].force = c2[i];
            aos[i].num_xy_bonds = c3[i];
            aos[i].num_z_bonds = c4[i];
            aos[i].num_stem_bonds = c5[i];
            aos[i].cycle = c6[i];
            aos[i].diff_noise_factor = c7[i];
            aos[i].dead_ticks = c8[i];
            aos[i].contact_inhibited_ticks = c9[i];
            aos[i].motility = c10[i];
            aos[i].dir = c11[i];
            aos[i].movement = c12[i];
        }
        std::free(c0);
        std::free(c1);
        std::free(c2);
        std::free(c3);
        std::free(c4);
        std::free(c5);
        std::free(c6);
        std::free(c7);
        std::free(c8);
        std::free(c9);
        std::free(c10);
        std::free(c11);
        std::free(c12);
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
        *DYN_ARRAY_PLACE(&agents.agents_Keratinocyte, Keratinocyte) = ([&]() { Keratinocyte abl_a; abl_a.type = abl_G.K_TYPE_STEM; abl_a.pos = random_5(abl_G, abl_R, float3_create(abl_G.SURFACE_WIDTH, abl_G.SURFACE_WIDTH, 50)); abl_a.force = float3_fill(0); abl_a.num_xy_bonds = 0; abl_a.num_z_bonds = 0; abl_a.num_stem_bonds = 0; abl_a.cycle = start_new_cycle_position(abl_G, abl_R, abl_G.K_TYPE_STEM); abl_a.diff_noise_factor = abl_random(abl_R, 0.9, 1.1); abl_a.dead_ticks = 0; abl_a.contact_inhibited_ticks = 0; abl_a.motility = abl_random(abl_R, 0, 0.5); abl_a.dir = 0.0; abl_a.movement = 0.0; return abl_a; }());
    }
    abl_simulate(abl_G.num_timesteps);
    return 0;
}
#else
#endif

}  // namespace abl_model_keratinocyte

#ifndef ABL_PERSIST
extern "C" const abl_model_desc *abl_model_desc_keratinocyte(void) {
    return &abl_model_keratinocyte::abl_desc;
}
#endif

#if defined(ABL_STANDALONE_MAIN) && !defined(ABL_PERSIST)
extern "C" const abl_model_desc *const abl_builtin_models[] = {
    &abl_model_keratinocyte::abl_desc, nullptr};
int main() { return abl_model_keratinocyte::abl_main(); }
#endif
