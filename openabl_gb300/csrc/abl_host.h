/* Host runtime for programs generated by `-b cuda`.
 *
 * The generated main() builds the initial population on the host exactly as
 * the `c` backend's program does and writes results with save(), so this
 * header offers the same host-side API as the reference runtime
 * (asset/c/libabl.h): the growable `dyn_array` with DYN_ARRAY_* accessors
 * (libabl.h:11-57), the sequential random_float / random_int generator with
 * its fixed seed (libabl.c:8-39), the run-time type tables and save() in the
 * JSON layout of libabl.c:46-124.  It is written for this project; only the
 * interface and the output format are the reference's. */
#ifndef ABL_HOST_H
#define ABL_HOST_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  void *values;
  size_t len;
  size_t cap;
} dyn_array;

#define DYN_ARRAY_GET(ary, elem_type, idx) (&((elem_type *) (ary)->values)[idx])
#define DYN_ARRAY_PLACE(ary, elem_type) ((elem_type *) dyn_array_place(ary, sizeof(elem_type)))
#define DYN_ARRAY_CREATE_FIXED(elem_type, len) dyn_array_create_fixed(sizeof(elem_type), len)
#define DYN_ARRAY_COPY_FIXED(elem_type, other) dyn_array_copy_fixed(sizeof(elem_type), other)

dyn_array dyn_array_create_fixed(size_t elem_size, size_t len);
dyn_array dyn_array_copy_fixed(size_t elem_size, const dyn_array *other);
void *dyn_array_place(dyn_array *ary, size_t elem_size);
void dyn_array_clean(dyn_array *ary);

/* Host RNG; `abl_host_use_float` selects the float or double variant of
 * random_float (the generated file passes its abl_float width). */
double random_float_d(double min, double max);
float random_float_f(float min, float max);
int random_int(int min, int max);
void abl_host_rng_reset(void);
/* The xorshift128+ state, to hand the stream to the device and back. */
void abl_host_rng_get(uint64_t state[2]);
void abl_host_rng_set(const uint64_t state[2]);

typedef enum {
  TYPE_END,
  TYPE_BOOL,
  TYPE_INT,
  TYPE_FLOAT,
  TYPE_STRING,
  TYPE_FLOAT2,
  TYPE_FLOAT3,
} type_id;

typedef struct {
  type_id type;
  unsigned offset;
  const char *name;
  bool is_pos;
} type_info;

typedef struct {
  const type_info *info;
  unsigned offset;
  const char *name;
} agent_info;

typedef enum {
  SAVE_JSON,
  SAVE_FLAME_XML,
  SAVE_FLAMEGPU_XML,
} save_type;

/* Writes every agent to `path` as JSON (SAVE_JSON, the format the `c`
 * backend's programs write) or FLAME / FLAMEGPU XML, as the reference
 * runtime's save() (asset/c/libabl.c:46-231).  `float_bytes` is
 * sizeof(abl_float) of the generated program.  Returns 0, or -1 (with a
 * message on stderr) when the file cannot be written or `type` is unknown. */
int abl_save(void *agents, const agent_info *info, const char *path, save_type type,
             int float_bytes);

#ifdef __cplusplus
}
#endif

#endif
