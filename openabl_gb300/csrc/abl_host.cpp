// Host runtime for programs generated by `-b cuda` (see abl_host.h).
#include "abl_host.h"

#include <climits>
#include <cstdlib>
#include <cstring>
#include <cstdio>

extern "C" {

dyn_array dyn_array_create_fixed(size_t elem_size, size_t len) {
  dyn_array a;
  a.values = std::calloc(len ? len : 1, elem_size);
  a.len = len;
  a.cap = len;
  return a;
}

dyn_array dyn_array_copy_fixed(size_t elem_size, const dyn_array *other) {
  dyn_array a = dyn_array_create_fixed(elem_size, other->len);
  std::memcpy(a.values, other->values, elem_size * other->len);
  return a;
}

void *dyn_array_place(dyn_array *ary, size_t elem_size) {
  if (ary->len == ary->cap) {
    ary->cap = ary->cap ? ary->cap * 2 : 128;
    ary->values = std::realloc(ary->values, elem_size * ary->cap);
  }
  return (char *) ary->values + elem_size * ary->len++;
}

void dyn_array_clean(dyn_array *ary) {
  std::free(ary->values);
  ary->values = nullptr;
  ary->len = ary->cap = 0;
}

// xorshift128+ (Vigna) with the reference's fixed seed.
static uint64_t rng_state[2] = {0xdeadbeefull, 0xbeefdeadull};

void abl_host_rng_reset(void) {
  rng_state[0] = 0xdeadbeefull;
  rng_state[1] = 0xbeefdeadull;
}

void abl_host_rng_get(uint64_t state[2]) {
  state[0] = rng_state[0];
  state[1] = rng_state[1];
}

void abl_host_rng_set(const uint64_t state[2]) {
  rng_state[0] = state[0];
  rng_state[1] = state[1];
}

static uint64_t rng_next(void) {
  uint64_t s1 = rng_state[0];
  const uint64_t s0 = rng_state[1];
  rng_state[0] = s0;
  s1 ^= s1 << 23;
  rng_state[1] = s1 ^ s0 ^ (s1 >> 17) ^ (s0 >> 26);
  return rng_state[1] + s0;
}

// min + x / (2^64-1 scaled to the interval), evaluated in the program's
// float width like the reference's random_float.
double random_float_d(double min, double max) {
  uint64_t x = rng_next();
  return min + (double) x / ((double) UINT64_MAX / (max - min));
}

float random_float_f(float min, float max) {
  uint64_t x = rng_next();
  return min + (float) x / ((float) UINT64_MAX / (max - min));
}

int random_int(int min, int max) {
  unsigned n = (unsigned) (max - min + 1);
  if ((n & (n - 1)) == 0) return (int) (rng_next() & (n - 1));
  unsigned lim = UINT_MAX - UINT_MAX % n;
  unsigned x;
  do {
    x = (unsigned) rng_next();
  } while (x >= lim);
  return min + (int) (x % n);
}

static size_t record_size(const type_info *info) {
  while (info->type != TYPE_END) ++info;
  return info->offset;
}

static double read_float(const char *p, int fb) {
  if (fb == 4) return *(const float *) p;
  return *(const double *) p;
}

static void write_member_json(FILE *f, const char *agent, const type_info *m, int fb) {
  const char *p = agent + m->offset;
  switch (m->type) {
    case TYPE_BOOL: std::fputs(*(const bool *) p ? "true" : "false", f); break;
    case TYPE_INT: std::fprintf(f, "%d", *(const int *) p); break;
    case TYPE_FLOAT: std::fprintf(f, "%f", read_float(p, fb)); break;
    case TYPE_FLOAT2:
      std::fprintf(f, "[%f,%f]", read_float(p, fb), read_float(p + fb, fb));
      break;
    case TYPE_FLOAT3:
      std::fprintf(f, "[%f,%f,%f]", read_float(p, fb), read_float(p + fb, fb),
                   read_float(p + 2 * fb, fb));
      break;
    default: break;
  }
}

// FLAME / FLAMEGPU XML (asset/c/libabl.c:126-213): one <xagent> per agent
// with its type name and one element per member; vectors are split into
// <m_x>, <m_y>[, <m_z>]; for FLAMEGPU the position member is always written
// as <x>, <y>, <z> (z = 0.0 in 2D).  Booleans are written as integers.  The
// reference reads a bool member through an int pointer, i.e. together with
// the three bytes after it in the agent record; here the member's own value
// (0 or 1) is written, which is what the reference writes when those bytes
// are zero.
static void write_member_xml(FILE *f, const char *agent, const type_info *m, int fb,
                             bool for_gpu) {
  const char *p = agent + m->offset;
  const char *nm = m->name;
  if (for_gpu && m->is_pos && (m->type == TYPE_FLOAT2 || m->type == TYPE_FLOAT3)) {
    std::fprintf(f, "<x>%f</x>\n<y>%f</y>\n", read_float(p, fb), read_float(p + fb, fb));
    if (m->type == TYPE_FLOAT3) std::fprintf(f, "<z>%f</z>\n", read_float(p + 2 * fb, fb));
    else std::fputs("<z>0.0</z>\n", f);
    return;
  }
  switch (m->type) {
    case TYPE_BOOL: std::fprintf(f, "<%s>%d</%s>\n", nm, *(const bool *) p ? 1 : 0, nm); break;
    case TYPE_INT: std::fprintf(f, "<%s>%d</%s>\n", nm, *(const int *) p, nm); break;
    case TYPE_FLOAT: std::fprintf(f, "<%s>%f</%s>\n", nm, read_float(p, fb), nm); break;
    case TYPE_FLOAT2:
    case TYPE_FLOAT3: {
      const int comps = m->type == TYPE_FLOAT2 ? 2 : 3;
      const char axis[3] = {'x', 'y', 'z'};
      for (int c = 0; c < comps; c++)
        std::fprintf(f, "<%s_%c>%f</%s_%c>\n", nm, axis[c], read_float(p + c * fb, fb), nm,
                     axis[c]);
      break;
    }
    default: break;
  }
}

static void save_json(FILE *f, void *agents, const agent_info *info, int float_bytes) {
  std::fputs("{", f);
  for (const agent_info *a = info; a->name; a++) {
    if (a != info) std::fputs(",", f);
    const dyn_array *arr = (const dyn_array *) ((const char *) agents + a->offset);
    std::fprintf(f, "\"%s\":[", a->name);
    size_t rec = record_size(a->info);
    for (size_t i = 0; i < arr->len; i++) {
      if (i) std::fputs(",\n", f);
      const char *agent = (const char *) arr->values + rec * i;
      std::fputs("{", f);
      for (const type_info *m = a->info; m->type != TYPE_END; m++) {
        if (m != a->info) std::fputs(",", f);
        std::fprintf(f, "\"%s\":", m->name);
        write_member_json(f, agent, m, float_bytes);
      }
      std::fputs("}", f);
    }
    std::fputs("]", f);
  }
  std::fputs("}", f);
}

static void save_xml(FILE *f, void *agents, const agent_info *info, int float_bytes,
                     bool for_gpu) {
  std::fputs("<states>\n<itno>0</itno>\n", f);
  for (const agent_info *a = info; a->name; a++) {
    const dyn_array *arr = (const dyn_array *) ((const char *) agents + a->offset);
    const size_t rec = record_size(a->info);
    for (size_t i = 0; i < arr->len; i++) {
      const char *agent = (const char *) arr->values + rec * i;
      std::fprintf(f, "<xagent>\n<name>%s</name>\n", a->name);
      for (const type_info *m = a->info; m->type != TYPE_END; m++)
        write_member_xml(f, agent, m, float_bytes, for_gpu);
      std::fputs("</xagent>\n", f);
    }
  }
  std::fputs("</states>\n", f);
}

int abl_save(void *agents, const agent_info *info, const char *path, save_type type,
             int float_bytes) {
  if (type != SAVE_JSON && type != SAVE_FLAME_XML && type != SAVE_FLAMEGPU_XML) {
    std::fprintf(stderr, "save(): unknown output format %d\n", (int) type);
    return -1;
  }
  FILE *f = std::fopen(path, "w");
  if (!f) {
    std::fprintf(stderr, "save(): Count not open \"%s\" for writing\n", path);
    return -1;
  }
  if (type == SAVE_JSON) save_json(f, agents, info, float_bytes);
  else save_xml(f, agents, info, float_bytes, type == SAVE_FLAMEGPU_XML);
  return std::fclose(f) == 0 ? 0 : -1;
}

}  // extern "C"
