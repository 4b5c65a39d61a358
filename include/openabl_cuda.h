/* OpenABL CUDA runtime — C ABI (GB300, sm_103a).
 *
 * This is the device runtime behind the `-b cuda` backend.  The reference
 * `c` backend keeps the agent population in host arrays and runs every step
 * function in-process (src/backend/CPrinter.cpp:189-233; runtime
 * asset/c/libabl.{h,c}).  With `-b cuda` the generated program keeps host
 * initialisation and save() unchanged and hands the population to this
 * runtime, which owns all device memory and one CUDA stream per context:
 *
 *   abl_create    -> allocation of the agent arrays (CPrinter.cpp:278-293,
 *                    `struct agent_struct` with agents_X / agents_X_dbuf)
 *   abl_upload    -> the state built by main() before `simulate`
 *   abl_step/run  -> one / T iterations of the simulate loop
 *                    (CPrinter.cpp:189-233: per step function, double buffer
 *                    copy on first use, parallel loop, swap)
 *   abl_download  -> the state read by save() after `simulate`
 *                    (CPrinter.cpp:74-76, asset/c/libabl.c:215-231)
 *   abl_reduce    -> the sequential-step reductions count()/sum()
 *                    (builtins at src/main.cpp:65-130, lowered for FlameGPU
 *                    at src/backend/FlameGPUBackend.cpp:204-225)
 *   abl_last_exec_time -> getLastExecTime() (src/main.cpp:66)
 *   abl_save_state / abl_load_state -> save() (asset/c/libabl.c:46-124),
 *                    binary and lossless, plus the resume the reference lacks
 *   abl_set_serial_random -> the one xorshift128+ stream random() draws
 *                    from (asset/c/libabl.c:8-39), continued in steps
 *
 * Conventions: every call returns 0 or a negative ABL_E_* code (text via
 * abl_strerror); host buffers belong to the caller, device buffers to the
 * context; one host thread per context; contexts on separate streams may run
 * concurrently.  Agent state crosses the boundary as structure-of-arrays: one
 * column per member, members in declaration order, each column holding n
 * values of the member's type (bool = 1 byte, int = int32, float = double or
 * float under use_float, float2/float3 = 2/3 consecutive floats).
 */
#ifndef OPENABL_CUDA_H
#define OPENABL_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ABL_OK 0
#define ABL_E_INVALID -1     /* bad argument */
#define ABL_E_BUDGET -2      /* the HBM budget given to abl_create is exhausted */
#define ABL_E_CUDA -3        /* a CUDA runtime call failed */
#define ABL_E_TIMEOUT -4     /* a bounded device-side wait ran out */
#define ABL_E_NONFINITE -5   /* an agent position is NaN or infinite */
#define ABL_E_UNSUPPORTED -6 /* model feature not implemented by this runtime */
#define ABL_E_CAPACITY -7    /* agent capacity exceeded by runtime additions */
#define ABL_E_NOMODEL -8     /* unknown model name */
#define ABL_E_SCRATCH -9     /* larger than abl_step_noalloc's fixed scratch area */
#define ABL_E_IO -10         /* a state file could not be written, read or matched */

/* Member value types (match asset/c/libabl.h:181-189 type_id). */
#define ABL_T_BOOL 1
#define ABL_T_INT 2
#define ABL_T_FLOAT 3
#define ABL_T_FLOAT2 5
#define ABL_T_FLOAT3 6

typedef struct abl_ctx abl_ctx;
typedef struct abl_model_desc abl_model_desc;

/* ---- model lookup (models compiled into this library by `-b cuda`) ---- */

/* Returns the descriptor of a built-in model (e.g. "boids2d"), or NULL. */
const abl_model_desc *abl_model_lookup(const char *name);
/* Number of agent types / their names / members (for generic hosts). */
int abl_model_num_agent_types(const abl_model_desc *m);
const char *abl_model_agent_name(const abl_model_desc *m, int type_id);
int abl_model_num_members(const abl_model_desc *m, int type_id);
int abl_model_member(const abl_model_desc *m, int type_id, int member, const char **name,
                     int *value_type);
/* Bytes of the model's float type: 8, or 4 when generated with use_float
 * (LIBABL_USE_FLOAT, asset/c/libabl.h:59-63). */
int abl_model_float_bytes(const abl_model_desc *m);
/* Size of the model's globals block (its `param`/constant declarations). */
size_t abl_model_globals_size(const abl_model_desc *m);
/* Writes the compile-time values of the globals (the constants printed by
 * the code generator) into `out` (abl_model_globals_size bytes). */
int abl_model_globals_default(const abl_model_desc *m, void *out);
/* Offset and type of a named global inside the globals block. */
int abl_model_global(const abl_model_desc *m, const char *name, size_t *offset, int *value_type);

/* ---- context lifecycle ---- */

/* Creates a context for `model` with the default globals.  `hbm_budget`
 * bounds the device memory the context may allocate (0 = unbounded). */
int abl_create(const abl_model_desc *model, size_t hbm_budget, abl_ctx **out);
/* Replaces the globals block (must precede abl_upload). */
int abl_set_globals(abl_ctx *ctx, const void *globals, size_t size);
/* Uploads `n` agents of `type_id` from host SoA columns (see above). */
int abl_upload(abl_ctx *ctx, int type_id, const void *const *cols, size_t n);
/* Initialisation on the device instead of an upload (main()'s `add` loops
 * run as kernels; the reference builds the population on the host,
 * CPrinter.cpp:278-293, and has no counterpart).  abl_reserve sizes the
 * type's buffers for `n` agents and stores the device address of each
 * member's column in dev_cols[member]; the caller fills them (and
 * synchronises its work with the device) before abl_commit, which makes the
 * double buffer a copy, as abl_upload does, and marks the type's binning
 * stale. */
int abl_reserve(abl_ctx *ctx, int type_id, size_t n, void **dev_cols);
int abl_commit(abl_ctx *ctx, int type_id);
/* Runs one / `timesteps` iterations of the simulate loop. */
int abl_step(abl_ctx *ctx);
int abl_run(abl_ctx *ctx, int timesteps);
/* Number of live agents of a type. */
int abl_count(abl_ctx *ctx, int type_id, size_t *n);
/* Copies the agents of `type_id` into host SoA columns of capacity *n;
 * sets *n to the number of agents. */
int abl_download(abl_ctx *ctx, int type_id, void *const *cols, size_t *n);
/* Sequential-step reductions (src/main.cpp:104-130; FlameGPU lowering at
 * src/backend/FlameGPUPrinter.cpp:204-225):
 *   ABL_REDUCE_COUNT     count(Type)          -> int
 *   ABL_REDUCE_SUM       sum(Type.member)     -> int for bool/int members (bools
 *                        sum to int), else the member's type; float members
 *                        are added in ascending agent order
 *   ABL_REDUCE_COUNT_EQ  count(Type.member, v) -> int; *out holds v on entry
 *                        (the member's type) and the count on return */
#define ABL_REDUCE_COUNT 0
#define ABL_REDUCE_SUM 1
#define ABL_REDUCE_COUNT_EQ 2
int abl_reduce(abl_ctx *ctx, int kind, int type_id, int member, void *out);
/* Seed of the counter-based generator behind random() in step functions
 * (Philox4x32-10 keyed by the seed; counter = agent index, step function,
 * timestep, draw).  Default 0. */
int abl_set_seed(abl_ctx *ctx, uint64_t seed);
/* Device time of the most recent timestep, in seconds: getLastExecTime()
 * inside a sequential step (src/backend/FlameGPUPrinter.cpp:246-249). */
int abl_last_timestep_time(abl_ctx *ctx, double *seconds);
/* Rows written by log_csv() in sequential steps ("%d"/"%f" comma-separated,
 * one row per call, as src/backend/FlameGPUPrinter.cpp:226-245 formats them).
 * abl_log_csv appends a row; abl_log_text copies the accumulated text. */
int abl_log_csv(abl_ctx *ctx, const char *fmt, ...);
int abl_log_text(abl_ctx *ctx, char *buf, size_t cap, size_t *len);
/* Wall time of the last abl_step/abl_run call, in seconds (device events). */
int abl_last_exec_time(abl_ctx *ctx, double *seconds);
/* Device memory currently held by the context, in bytes. */
int abl_memory_used(abl_ctx *ctx, size_t *bytes);
/* Number of kernel launches issued by the last abl_step/abl_run call. */
int abl_last_launch_count(abl_ctx *ctx, long *launches);
/* Per-step-function kernel timing with device events (for profiling; eager
 * timesteps only, so abl_run does not replay graphs while it is on). */
int abl_set_profiling(abl_ctx *ctx, int enable);
int abl_step_kernel_time(abl_ctx *ctx, int step, double *seconds, long *launches);
/* Ordered near loops gather each block's neighbour lists in shared memory;
 * with balancing on (the default) the block's agents are handed to its
 * threads in order of neighbour count, so a warp's loops have similar
 * lengths.  Results are identical either way. */
int abl_set_balance(abl_ctx *ctx, int enable);
/* How ordered near loops find their neighbours in ascending id: ABL_NEAR_AUTO
 * (default) picks per step; RUNS sorts each agent's neighbours from the
 * cells' own runs, ROWS (2D) merges three precomputed row lists per agent,
 * LISTS reads whole precomputed neighbourhood lists, BLOCK (2D, loops around
 * the step's own agents) has each thread block merge the row lists once per
 * cell in shared memory (falling back to ROWS for a block whose lists do not
 * fit).  Results are identical in every mode; this is a tuning and testing
 * control. */
#define ABL_NEAR_AUTO 0
#define ABL_NEAR_RUNS 1
#define ABL_NEAR_ROWS 2
#define ABL_NEAR_LISTS 3
#define ABL_NEAR_BLOCK 4
int abl_set_near_mode(abl_ctx *ctx, int mode);
/* A near loop around the step's own agent, over a type whose positions no
 * step function changes (nor adds or removes agents of), keeps each agent's
 * in-radius neighbour list from one binning to the next: found once after an
 * upload, read at every timestep (default on).  Results are identical either
 * way. */
int abl_set_near_cache(abl_ctx *ctx, int enable);
/* Sequential random numbers: random() inside step functions continues the
 * reference's single xorshift128+ stream (asset/c/libabl.c:8-39) from
 * `state`, in the order the reference program draws on one thread: step
 * functions in order, agents in index order.  Steps that draw run one agent
 * per launch, so this is a parity mode, not a fast one.  NULL turns it off
 * (counter-based streams).  abl_get_serial_random reads the state back. */
int abl_set_serial_random(abl_ctx *ctx, const uint64_t *state);
int abl_get_serial_random(abl_ctx *ctx, uint64_t *state);
/* Checkpoint and resume (the reference has no resume, and its save() prints
 * %f, which loses bits): abl_save_state writes the whole simulation state to
 * a binary file -- globals, timestep, random-number seed and sequential
 * state, and per agent type both buffers of every member (step functions
 * that do not write a member leave the double buffer's older value visible,
 * as the reference's agents_X_dbuf does).  abl_load_state restores it into a
 * context of the same model; the resumed run then equals the uninterrupted
 * one bit for bit.  ABL_E_IO: the file cannot be written or read, or holds
 * another model's state. */
int abl_save_state(abl_ctx *ctx, const char *path);
int abl_load_state(abl_ctx *ctx, const char *path);
int abl_destroy(abl_ctx *ctx);
const char *abl_strerror(int code);

/* ---- ensembles ----
 *
 * Many replicas of one model -- different agent counts, parameter points
 * (globals) and seeds -- run as one population over a segmented grid: each
 * timestep is one launch per phase for all replicas, replayed from a CUDA
 * graph.  Per replica the results equal those of a separate context.  Models
 * with runtime add/remove or a sequential step are not supported. */
typedef struct abl_ensemble abl_ensemble;
/* `globals`: replicas x globals_size bytes (NULL: defaults); `seeds`: one
 * random() seed per replica (NULL: 0). */
int abl_ensemble_create(const abl_model_desc *model, int replicas, const void *globals,
                        const uint64_t *seeds, size_t hbm_budget, abl_ensemble **out);
/* All replicas of one agent type at once: counts[r] agents of replica r,
 * columns concatenated replica after replica. */
int abl_ensemble_upload(abl_ensemble *e, int type_id, const size_t *counts,
                        const void *const *cols);
int abl_ensemble_run(abl_ensemble *e, int timesteps);
int abl_ensemble_download(abl_ensemble *e, int type_id, size_t *counts, void *const *cols);
/* Launch configuration: threads per block of the step kernels (32..128),
 * cell size as a multiple (>= 1) of the granularity, and whether threads visit
 * agents in cell order (1) or index order (0).  Results do not depend on it. */
int abl_ensemble_set_tuning(abl_ensemble *e, int block, double cell_factor, int visit_sorted);
/* Cells-per-block tiling of ordered 2D near loops when threads visit agents
 * in cell order: each thread block merges the neighbourhood lists of the run
 * of cells its agents fill once, in shared memory, holding up to `entries`
 * list entries (0: no block tiling, every agent merges its own rows; else a
 * multiple of 256 up to 4096).  A block whose cells need more falls back to
 * per-agent merging.  Results do not depend on it. */
int abl_ensemble_set_tiling(abl_ensemble *e, int entries);
/* The configuration in use (any pointer may be NULL). */
int abl_ensemble_get_tuning(abl_ensemble *e, int *block, double *cell_factor, int *visit_sorted,
                            int *tiling_entries);
/* Times every configuration -- block size, cell size factor, visiting order
 * and tiling -- for `trial_timesteps` timesteps, restores the state after
 * each trial and keeps the fastest (abl_ensemble_get_tuning reports the
 * tiling it chose). */
int abl_ensemble_autotune(abl_ensemble *e, int trial_timesteps, int *block, double *cell_factor,
                          int *visit_sorted);
int abl_ensemble_last_exec_time(abl_ensemble *e, double *seconds);
int abl_ensemble_last_launch_count(abl_ensemble *e, long *launches);
/* Persistent runs (enable = 1): abl_ensemble_run executes all its timesteps
 * -- every binning phase and step function of every replica -- in ONE
 * cooperative kernel launch of as many blocks as the device holds at once,
 * the phases separated by grid-wide barriers.  Each barrier wait gives up
 * after a time limit (4 s by default), and the run then returns
 * ABL_E_TIMEOUT; the replicas' state is then undefined until the next
 * abl_ensemble_upload.  Results equal those of the per-phase launches bit
 * for bit.  The launch holds every SM until the run ends, so work on other
 * streams waits for it.
 * ABL_E_UNSUPPORTED for models without an ensemble form.  The replicas'
 * timestep pattern must repeat with period two after the first (every model
 * whose steps all run each timestep does). */
int abl_ensemble_set_persistent(abl_ensemble *e, int enable);
/* Blocks of the last persistent launch (0 before the first). */
int abl_ensemble_persistent_blocks(abl_ensemble *e, int *blocks);
/* Durations of the first phases of the last persistent run, in order (the
 * time between the ends of consecutive phases as block 0 saw them: the
 * binning phases of the first timestep, its step functions, then the next
 * timestep's): up to `cap` of them, *count set to how many. */
int abl_ensemble_phase_times(abl_ensemble *e, double *seconds, int cap, int *count);
int abl_ensemble_destroy(abl_ensemble *e);

/* ---- serving: continuous batching of simulation jobs ----
 *
 * No counterpart in the reference, whose programs run one simulation per
 * process.  A server runs submitted simulation jobs concurrently: a job is
 * admitted as soon as one of `slots` workers is free and its estimated
 * device memory fits in what is left of `hbm_budget` (0: 90% of free
 * memory); each running job has its own context and stream (small jobs of
 * one model share an ensemble, abl_server_set_batching), so the work of all
 * running jobs overlaps on the device, and queued jobs start as soon as
 * running ones release their slot and memory.  State stays on the device for
 * the whole job; results are kept in host memory until released. */
typedef struct abl_server abl_server;
typedef struct {
  const abl_model_desc *model;
  const void *globals;          /* NULL: the model's defaults */
  uint64_t seed;                /* random() seed */
  int timesteps;
  const size_t *counts;         /* agents per type */
  const void *const *const *cols; /* per type: host SoA columns (copied at submit) */
} abl_job_desc;
int abl_server_create(int slots, size_t hbm_budget, abl_server **out);
int abl_server_submit(abl_server *s, const abl_job_desc *job, long *job_id);
/* Blocks until the job has finished (ABL_E_TIMEOUT after timeout_s). */
int abl_server_wait(abl_server *s, long job_id, double timeout_s);
/* status: 0 queued, 1 running, 2 done, < 0 failed with that ABL_E_* code;
 * times[4]: submit, admission and completion (seconds, steady clock) and the
 * device time of its timesteps. */
int abl_server_job_info(abl_server *s, long job_id, int *status, double *times);
/* Final population of one agent type (like abl_download). */
int abl_server_result(abl_server *s, long job_id, int type_id, void *const *cols, size_t *n);
int abl_server_release(abl_server *s, long job_id);
int abl_server_stats(abl_server *s, int *queued, int *running, size_t *bytes_in_use);
/* Batching of small jobs (default: up to 64 jobs of at most 65,536 agents
 * each): a worker that admits such a job of a model with an ensemble form
 * also admits the queued small jobs of the same model whose memory fits, and
 * runs them as the replicas of one ensemble in its slot (one launch per
 * phase for all of them), each job completing when its own timestep count
 * is reached.
 * Results are those of each job run alone.  max_jobs = 1 turns it off. */
int abl_server_set_batching(abl_server *s, int max_jobs, long max_agents);
/* Runs the queued jobs to completion, then stops the workers. */
int abl_server_destroy(abl_server *s);

/* ---- allocation-free timestep ----
 *
 * No counterpart in the reference (whose `c` backend never touches a GPU).
 * For callers that cannot allocate device memory while they run -- code
 * embedded in another framework's memory pool or allocator, or loops that
 * must not allocate once started: runs ONE timestep of a model with one
 * agent type and one step function on device buffers the caller owns
 * (SoA columns as above, device pointers): reads `in_cols`, writes
 * `out_cols` (members the step does not always write keep the values
 * already in `out_cols`, like the reference's double buffer).  `globals` is
 * the model's globals block on the host; `stream` is a cudaStream_t (NULL for
 * the default stream).  The call is synchronous.
 *
 * It calls no cudaMalloc/cudaFree: its temporaries live in one static device
 * array of ABL_NOALLOC_SCRATCH_BYTES, which every GPU that loads this library
 * holds until the process exits.  Limits: at most ABL_NOALLOC_MAX_AGENTS
 * agents and ABL_NOALLOC_MAX_CELLS grid cells, and everything must fit the
 * array; larger problems return ABL_E_SCRATCH without touching the GPU.  In
 * 3D the neighbourhood lists take about 300 bytes per agent, so there the
 * array runs out near 90,000 agents.  Models whose step calls random(),
 * removeCurrent() or add(), and models with a sequential step, return
 * ABL_E_UNSUPPORTED before any GPU work.  The
 * first call on a device, with that device current, looks up the array's
 * address (cudaGetSymbolAddress) and sets up host bookkeeping; make it
 * before any stream capture.  All calls share the array: calls that overlap
 * on the GPU race and must be serialised by the caller. */
#define ABL_NOALLOC_MAX_AGENTS 131072
#define ABL_NOALLOC_MAX_CELLS 131072
#define ABL_NOALLOC_SCRATCH_BYTES (32u << 20)
int abl_step_noalloc(const abl_model_desc *model, const void *globals, size_t globals_size,
                     const void *const *in_cols, void *const *out_cols, size_t n, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* OPENABL_CUDA_H */
