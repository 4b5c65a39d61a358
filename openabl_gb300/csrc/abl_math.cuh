// Vector types and math for generated code, usable on host and device.
//
// Included INSIDE a generated model's namespace after
//   typedef double abl_float;   (or float under use_float)
// so that the generated code can use the same names and the same arithmetic
// as the reference runtime's header (asset/c/libabl.h:59-175): float2/float3
// are structs of abl_float (shadowing CUDA's own float2/float3 inside the
// namespace), operations are component-wise, and length/dist take sqrtf of
// the abl_float sum of squares, which rounds that sum to float first.  The
// file is compiled with -fmad=false so that no multiply-add is contracted,
// matching the reference build (gcc -std=c99, no FP contraction).
// No include guard: it is included once per model namespace.

struct float2 {
  abl_float x;
  abl_float y;
};

struct float3 {
  abl_float x;
  abl_float y;
  abl_float z;
};

__host__ __device__ static inline abl_float min(abl_float x, abl_float y) { return fmin(x, y); }
__host__ __device__ static inline abl_float max(abl_float x, abl_float y) { return fmax(x, y); }

__host__ __device__ static inline float2 float2_create(abl_float x, abl_float y) {
  float2 r = {x, y};
  return r;
}
__host__ __device__ static inline float2 float2_fill(abl_float x) { return float2_create(x, x); }
// Sums and differences of components; FP64 ones on the device go through
// abl::dadd / abl::dsub (the same correctly rounded results).
__host__ __device__ static inline abl_float abl_add(abl_float a, abl_float b) {
#ifdef __CUDA_ARCH__
  if (sizeof(abl_float) == sizeof(double)) return (abl_float) abl::dadd((double) a, (double) b);
#endif
  return a + b;
}
__host__ __device__ static inline abl_float abl_sub(abl_float a, abl_float b) {
#ifdef __CUDA_ARCH__
  if (sizeof(abl_float) == sizeof(double)) return (abl_float) abl::dsub((double) a, (double) b);
#endif
  return a - b;
}
__host__ __device__ static inline float2 float2_add(float2 a, float2 b) {
  return float2_create(abl_add(a.x, b.x), abl_add(a.y, b.y));
}
__host__ __device__ static inline float2 float2_sub(float2 a, float2 b) {
  return float2_create(abl_sub(a.x, b.x), abl_sub(a.y, b.y));
}
__host__ __device__ static inline float2 float2_mul_scalar(float2 a, abl_float s) {
  return float2_create(a.x * s, a.y * s);
}
__host__ __device__ static inline float2 float2_div_scalar(float2 a, abl_float s) {
  return float2_create(a.x / s, a.y / s);
}
// Division by an int (e.g. a neighbour count): the same value as converting
// the int and dividing, computed on the device by abl::div_int in FP64.
// A template on exactly `int`, so calls with a floating divisor keep the
// overload above.
__host__ __device__ static inline abl_float abl_div_count(abl_float a, int n) {
#ifdef __CUDA_ARCH__
  if (sizeof(abl_float) == sizeof(double)) return (abl_float) abl::div_int((double) a, n);
#endif
  return a / (abl_float) n;
}
template <typename I, typename std::enable_if<std::is_same<I, int>::value, int>::type = 0>
__host__ __device__ static inline float2 float2_div_scalar(float2 a, I s) {
  return float2_create(abl_div_count(a.x, s), abl_div_count(a.y, s));
}
__host__ __device__ static inline bool float2_equals(float2 a, float2 b) {
  return a.x == b.x && a.y == b.y;
}
__host__ __device__ static inline bool float2_not_equals(float2 a, float2 b) {
  return a.x != b.x || a.y != b.y;
}

__host__ __device__ static inline float3 float3_create(abl_float x, abl_float y, abl_float z) {
  float3 r = {x, y, z};
  return r;
}
__host__ __device__ static inline float3 float3_fill(abl_float x) { return float3_create(x, x, x); }
__host__ __device__ static inline float3 float3_add(float3 a, float3 b) {
  return float3_create(abl_add(a.x, b.x), abl_add(a.y, b.y), abl_add(a.z, b.z));
}
__host__ __device__ static inline float3 float3_sub(float3 a, float3 b) {
  return float3_create(abl_sub(a.x, b.x), abl_sub(a.y, b.y), abl_sub(a.z, b.z));
}
__host__ __device__ static inline float3 float3_mul_scalar(float3 a, abl_float s) {
  return float3_create(a.x * s, a.y * s, a.z * s);
}
__host__ __device__ static inline float3 float3_div_scalar(float3 a, abl_float s) {
  return float3_create(a.x / s, a.y / s, a.z / s);
}
template <typename I, typename std::enable_if<std::is_same<I, int>::value, int>::type = 0>
__host__ __device__ static inline float3 float3_div_scalar(float3 a, I s) {
  return float3_create(abl_div_count(a.x, s), abl_div_count(a.y, s), abl_div_count(a.z, s));
}
__host__ __device__ static inline bool float3_equals(float3 a, float3 b) {
  return a.x == b.x && a.y == b.y && a.z == b.z;
}
__host__ __device__ static inline bool float3_not_equals(float3 a, float3 b) {
  return a.x != b.x || a.y != b.y || a.z != b.z;
}

__host__ __device__ static inline abl_float dot_float2(float2 a, float2 b) {
  return a.x * b.x + a.y * b.y;
}
__host__ __device__ static inline abl_float dot_float3(float3 a, float3 b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
__host__ __device__ static inline abl_float length_float2(float2 v) {
  return sqrtf((float) (v.x * v.x + v.y * v.y));
}
__host__ __device__ static inline abl_float length_float3(float3 v) {
  return sqrtf((float) (v.x * v.x + v.y * v.y + v.z * v.z));
}
__host__ __device__ static inline abl_float dist_float2(float2 a, float2 b) {
  return length_float2(float2_sub(a, b));
}
__host__ __device__ static inline abl_float dist_float3(float3 a, float3 b) {
  return length_float3(float3_sub(a, b));
}
__host__ __device__ static inline float2 normalize_float2(float2 v) {
  return float2_div_scalar(v, length_float2(v));
}
__host__ __device__ static inline float3 normalize_float3(float3 v) {
  return float3_div_scalar(v, length_float3(v));
}

// Host RNG in the program's float width (asset/c/libabl.c:19-24).
static inline abl_float abl_random_float(abl_float lo, abl_float hi) {
  if (sizeof(abl_float) == sizeof(float)) return (abl_float) random_float_f((float) lo, (float) hi);
  return (abl_float) random_float_d((double) lo, (double) hi);
}

// random() / randomInt(): the sequential host stream in main(), the
// counter-based stream (abl::rng) inside step kernels.
__host__ __device__ static inline abl_float abl_random(abl::rng &R, abl_float lo, abl_float hi) {
#ifdef __CUDA_ARCH__
  return R.uniform<abl_float>(lo, hi);
#else
  (void) R;
  return abl_random_float(lo, hi);
#endif
}
__host__ __device__ static inline int abl_random_int(abl::rng &R, int lo, int hi) {
#ifdef __CUDA_ARCH__
  return R.uniform_int(lo, hi);
#else
  (void) R;
  return random_int(lo, hi);
#endif
}
