/* Contract between code emitted by the `-b cuda` backend and the runtime.
 *
 * A generated model file describes its agent types (from the AST's
 * AgentDeclaration list, CPrinter.cpp:250-265 prints the same information as
 * `type_info` tables), its globals (the folded `param`/constant
 * declarations, CPrinter.cpp:305-307), its environment (EnvironmentDeclaration,
 * src/AnalysisVisitor.cpp:474-538) and its step functions in simulate order
 * (SimulateStatement::stepFuncDecls, CPrinter.cpp:196).  Each step function
 * comes with a host launcher that runs its kernel on a stream.
 */
#ifndef ABL_MODEL_H
#define ABL_MODEL_H

#include <stddef.h>
#include <stdint.h>
#include <cuda_runtime.h>

#include "openabl_cuda.h"

#define ABL_MAX_MEMBERS 16

typedef struct {
  const char *name;
  int value_type;     /* ABL_T_* */
  int components;     /* 1, 2 or 3 */
  int scalar_bytes;   /* bytes of one component (1, 4 or 8) */
  int is_position;
} abl_member_desc;

typedef struct {
  const char *name;
  int num_members;
  const abl_member_desc *members;
  int position_member; /* index of the `position` member, -1 if none */
  int dim;             /* 2 or 3 when a position member exists */
} abl_agent_desc;

typedef struct {
  const char *name;
  int value_type;
  size_t offset;
} abl_global_desc;

/* Binned view of the neighbour type, filled by the runtime for a step
 * function that contains a `near` loop.  All pointers are device pointers;
 * arrays indexed by "slot" are in (cell, agent id) order. */
typedef struct {
  int dim;
  int ordered;              /* 1: per-cell neighbourhood lists in ascending id order */
  int range;                /* cells searched on each side of the agent's cell */
  int nx, ny, nz;           /* grid dimensions */
  double lo[3];             /* grid origin */
  double inv_cell;          /* 1 / cell size */
  double radius;            /* value of the near() radius expression */
  long n;                   /* agents of the neighbour type */
  const int *cell_start;    /* ncells + 1 */
  const int *order;         /* slot -> agent id */
  const float *posf;        /* slot -> position rounded to float (dim per slot) */
  const int *nb_off;        /* ordered mode: cell -> offset into nb_list (ncells + 1) */
  const int *nb_list;       /* ordered mode: slots, ascending agent id per cell */
  const int *row_off;       /* row lists: cell -> offset into rows (ncells + 1) */
  const int4 *rows;         /* row lists: (id, slot, float x, float y) of the cells c-1..c+1
                               along x, ascending id */
  const float *amax;        /* max |coordinate| over neighbour and query agents */
  const void *cols[ABL_MAX_MEMBERS]; /* slot-ordered copies of the members the loop reads */
  const int *cell_of;       /* agent -> cell when the step's agents are the binned ones, else NULL */
  long cell_base;           /* cell_of values are cell_base + cell index of this view */
  int balance;              /* presorted mode: hand a block's agents to threads by neighbour count */
  int cap;                  /* presorted mode: neighbours held per agent in shared memory */
  int block_cap;            /* row lists, agents visited in slot order: entries of the
                               per-block neighbourhood lists in shared memory (0: off) */
  const int *ncache_off;    /* neighbour lists kept across timesteps (NULL: none): query
                               agent i's in-radius neighbours are entries off[i] .. off[i+1]
                               of ncache_list, in ascending index for ordered loops; `cols`
                               and `posf` are then indexed by agent, not by slot */
  const void *ncache_list;  /* int32 agent indices, or with ncache_narrow int16 offsets
                               from the query agent's index */
  int ncache_narrow;
  int cell_f32;             /* query cells may be computed in FP32 (as the binning does) */
  /* mixed precision: slot-ordered float copies of the members a loop sums in
     FP32, and the low part of the position, (float) (pos - (double) posf) */
  const void *fcols[ABL_MAX_MEMBERS];
  const float *poslo;
} abl_near_view;

/* Everything a generated step launcher needs. */
typedef struct {
  long n;                            /* agents of the step's type */
  void *in_cols[ABL_MAX_MEMBERS];    /* current buffer, per member */
  void *out_cols[ABL_MAX_MEMBERS];   /* double buffer, per member */
  const int *visit_order;            /* thread -> agent id (NULL: identity) */
  const void *globals;               /* host copy of the globals block */
  int *error;                        /* device error word */
  abl_near_view near;                /* valid when the step has a near loop */
  int block;                         /* threads per block chosen by the runtime */
  size_t smem;                       /* dynamic shared memory per block */
  /* runtime removal / addition (steps that call removeCurrent() / add()) */
  uint8_t *removed;                  /* per agent: 1 when the agent removed itself */
  uint8_t *child_flag;               /* per agent: 1 when it created a child */
  void *child_cols[ABL_MAX_MEMBERS]; /* members of the created child, by parent index */
  /* counter-based random numbers for random() in step functions */
  uint64_t seed;
  long timestep;
  int step_index;
  /* members the kernel need not store: the step only ever copies them from
     `in`, and the double buffer already holds the same values */
  uint32_t skip_store;
  /* sequential random numbers: the xorshift128+ state (device), or NULL */
  unsigned long long *serial_rng;
} abl_step_launch;

typedef int (*abl_step_launch_fn)(const abl_step_launch *launch, cudaStream_t stream);

/* Ensemble launch: the agents of many replicas of one model in one launch.
 * Agent i belongs to replica replica[i]; that replica's globals block is
 * globals + replica[i] * globals_size and its binned neighbour view is
 * views[replica[i]] (device arrays).  Column and slot indices are global. */
typedef struct {
  long n;                            /* agents of the step's type, all replicas */
  void *in_cols[ABL_MAX_MEMBERS];
  void *out_cols[ABL_MAX_MEMBERS];
  const int *visit_order;
  const int *replica;                /* agent -> replica */
  const void *globals;               /* device: replicas x globals_size bytes */
  const abl_near_view *views;        /* device: one view per replica */
  const long *agent_base;            /* device: first agent of each replica */
  const uint64_t *seeds;             /* device: random() seed per replica */
  long timestep;
  int step_index;
  int block;
  size_t smem;                       /* dynamic shared memory per block */
} abl_ens_launch;

typedef int (*abl_ens_launch_fn)(const abl_ens_launch *launch, cudaStream_t stream);

/* Persistent ensemble kernel: runs the program `prog` (device memory, an
 * abl::persist_prog of abl_persist.cuh) in one cooperative launch of as many
 * blocks of `block` threads as are co-resident on the device with `smem`
 * bytes of dynamic shared memory each, or *grid blocks when that is
 * positive and fewer; *grid receives the block count.  With prog == NULL it
 * only computes *grid.  `error` is the device error word for non-finite
 * positions. */
typedef int (*abl_persist_launch_fn)(const void *prog, int *error, int block, size_t smem,
                                     int *grid, cudaStream_t stream);
typedef double (*abl_globals_fn)(const void *globals);
typedef void (*abl_env_fn)(const void *globals, double *min3, double *max3);

typedef struct {
  const char *name;
  int agent_type;              /* type of the step's `in -> out` parameter */
  int near_type;               /* type iterated by the near loop, -1 if none */
  int ordered;                 /* the near body depends on the visiting order */
  abl_globals_fn radius;       /* value of the near radius expression */
  uint32_t near_members;       /* bitmask of neighbour members read in the loop */
  uint32_t out_written;        /* bitmask of members always written to `out` */
  abl_step_launch_fn launch;
  int uses_remove;             /* the body may call removeCurrent() */
  int add_type;                /* agent type created by add() in the body, -1 if none */
  int out_copy;                /* `out` starts as a copy of `in` */
  abl_ens_launch_fn launch_ens; /* ensemble variant (NULL: not supported) */
  int uses_rng;                 /* the body draws random numbers */
  int presorted;                /* ordered near loop served from per-block sorted lists */
  uint32_t out_changed;         /* bitmask of members the body may set to anything but the
                                   agent's own `in` value (`out.m = in.m` does not count) */
  int near_cacheable;           /* one near loop, centred on the step's own agent */
  uint32_t near_members_f32;    /* mixed precision: neighbour members summed from float copies */
  int near_pos_lo;              /* mixed precision: the loop sums position offsets (needs the
                                   position's low part) */
} abl_step_desc;

/* Host function run after every timestep: the `sequential step`. */
typedef int (*abl_seq_step_fn)(abl_ctx *ctx, const void *globals);

/* Called by the sequential step's builtins (count, sum, getLastExecTime)
 * when their runtime call fails: the first such code is what the timestep
 * returns once the sequential step has finished. */
#ifdef __cplusplus
extern "C"
#endif
void abl_seq_record_error(abl_ctx *ctx, int code);

struct abl_model_desc {
  const char *name;
  int num_agent_types;
  const abl_agent_desc *agents;
  int num_steps;
  const abl_step_desc *steps;   /* in simulate order */
  size_t globals_size;
  const void *globals_default;
  int num_globals;
  const abl_global_desc *globals;
  int env_dim;                   /* 0 when there is no environment */
  abl_env_fn env_bounds;
  abl_globals_fn granularity;    /* cell size before the safety margin */
  int uses_float;                /* built with use_float */
  abl_seq_step_fn seq_step;      /* NULL when the simulation has none */
  abl_persist_launch_fn launch_ens_persist; /* NULL when the model has no ensemble form */
};

#endif /* ABL_MODEL_H */
