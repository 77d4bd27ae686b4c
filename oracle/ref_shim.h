/*
 * ref_shim.h -- the handful of OpenCL C built-ins that the reference's
 * kernels use, written as plain C++ so that the reference's own kernel
 * source compiles on the host (test infrastructure; see make_ref.py).
 *
 * What it provides: 3-component vectors (float3/double3/uint3) with
 * component-wise arithmetic and scalar broadcasting, vload3/vstore3,
 * dot/length/clamp, the float/double math overloads (so that pow(float, 6)
 * stays single precision as in OpenCL C), work-item ids from a
 * thread-local index set by the host loop, and no-op barriers.  Address
 * space qualifiers are erased by macros defined in the generated file.
 *
 * The file has no include guard and no namespace: make_ref.py includes it
 * INSIDE each generated namespace (after <math.h>, <stddef.h>, <stdint.h>
 * and <type_traits>), so that unqualified calls in the kernel source find
 * these overloads first, as OpenCL C would, and never the <math.h> ones.
 *
 * float->uint conversion saturates (negative and NaN -> 0), the GPU rule;
 * C++ leaves out-of-range conversion undefined.
 */

typedef unsigned int uint;

template <typename T>
struct vec3 {
    T x, y, z;
    vec3 &operator+=(const vec3 &o) { x += o.x; y += o.y; z += o.z; return *this; }
    vec3 &operator-=(const vec3 &o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    template <typename S> vec3 &operator*=(S s) { T t = (T)s; x *= t; y *= t; z *= t; return *this; }
    template <typename S> vec3 &operator/=(S s) { T t = (T)s; x /= t; y /= t; z /= t; return *this; }
};
typedef vec3<float> float3;
typedef vec3<double> double3;
typedef vec3<uint> uint3;

#define CLSHIM_SCALAR(S) typename std::enable_if<std::is_arithmetic<S>::value, int>::type = 0
template <typename T> inline vec3<T> operator+(vec3<T> a, vec3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename T> inline vec3<T> operator-(vec3<T> a, vec3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename T> inline vec3<T> operator-(vec3<T> a) { return {-a.x, -a.y, -a.z}; }
template <typename T> inline vec3<T> operator*(vec3<T> a, vec3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <typename T> inline vec3<T> operator/(vec3<T> a, vec3<T> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
/* vector (op) scalar: the scalar is converted to the element type */
template <typename T, typename S, CLSHIM_SCALAR(S)> inline vec3<T> operator*(vec3<T> a, S s) { T t = (T)s; return {a.x * t, a.y * t, a.z * t}; }
template <typename T, typename S, CLSHIM_SCALAR(S)> inline vec3<T> operator*(S s, vec3<T> a) { T t = (T)s; return {t * a.x, t * a.y, t * a.z}; }
template <typename T, typename S, CLSHIM_SCALAR(S)> inline vec3<T> operator/(vec3<T> a, S s) { T t = (T)s; return {a.x / t, a.y / t, a.z / t}; }
template <typename T, typename S, CLSHIM_SCALAR(S)> inline vec3<T> operator+(vec3<T> a, S s) { T t = (T)s; return {a.x + t, a.y + t, a.z + t}; }
template <typename T, typename S, CLSHIM_SCALAR(S)> inline vec3<T> operator-(vec3<T> a, S s) { T t = (T)s; return {a.x - t, a.y - t, a.z - t}; }
#undef CLSHIM_SCALAR

template <typename A> inline uint sat_uint(A v) {
    double d = (double)v;
    if (!(d > 0)) return 0u;
    if (d >= 4294967296.0) return 0xFFFFFFFFu;
    return (uint)d;
}
/* (float3)(a,b,c), (double3)(...), (uint3)(...) literals are rewritten to
 * these calls by the generator. */
template <typename A, typename B, typename C> inline float3 make_float3(A a, B b, C c) { return {(float)a, (float)b, (float)c}; }
template <typename A, typename B, typename C> inline double3 make_double3(A a, B b, C c) { return {(double)a, (double)b, (double)c}; }
template <typename A, typename B, typename C> inline uint3 make_uint3(A a, B b, C c) { return {sat_uint(a), sat_uint(b), sat_uint(c)}; }

template <typename P> inline vec3<typename std::remove_cv<P>::type> vload3(size_t i, P *p) {
    return {p[3 * i], p[3 * i + 1], p[3 * i + 2]};
}
template <typename T> inline void vstore3(vec3<T> v, size_t i, T *p) { p[3 * i] = v.x; p[3 * i + 1] = v.y; p[3 * i + 2] = v.z; }

inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double dot(double3 a, double3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(float3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
inline double length(double3 a) { return ::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline uint3 clamp(uint3 v, uint3 lo, uint3 hi) {
    uint3 r;
    r.x = v.x < lo.x ? lo.x : (v.x > hi.x ? hi.x : v.x);
    r.y = v.y < lo.y ? lo.y : (v.y > hi.y ? hi.y : v.y);
    r.z = v.z < lo.z ? lo.z : (v.z > hi.z ? hi.z : v.z);
    return r;
}

inline float pow(float a, float b) { return powf(a, b); }
inline double pow(double a, double b) { return ::pow(a, b); }
inline float fabs(float a) { return fabsf(a); }
inline double fabs(double a) { return ::fabs(a); }
inline float sqrt(float a) { return sqrtf(a); }
inline double sqrt(double a) { return ::sqrt(a); }
inline float rsqrt(float a) { return 1.0f / sqrtf(a); }
inline double rsqrt(double a) { return 1.0 / ::sqrt(a); }
inline float atan(float a) { return atanf(a); }
inline double atan(double a) { return ::atan(a); }
inline float cos(float a) { return cosf(a); }
inline double cos(double a) { return ::cos(a); }
inline float sin(float a) { return sinf(a); }
inline double sin(double a) { return ::sin(a); }

/* work-item functions: the host loop sets the global id before each call
 * (a 3-D launch, as populate_position_cuboid needs, also sets the y and z
 * ids and the work dimension) */
static thread_local size_t g_global_id;
static thread_local size_t g_global_id_yz[2];
static thread_local uint g_work_dim = 1;
inline size_t get_global_id(uint d) { return d == 0 ? g_global_id : (d < 3 ? g_global_id_yz[d - 1] : 0); }
inline size_t get_local_id(uint) { return 0; }
inline size_t get_local_size(uint) { return 1; }
inline size_t get_group_id(uint) { return 0; }
inline uint get_work_dim() { return g_work_dim; }
enum { CLK_LOCAL_MEM_FENCE = 1, CLK_GLOBAL_MEM_FENCE = 2 };
inline void barrier(int) {}
inline uint atomic_inc(uint *p) { return (*p)++; }
