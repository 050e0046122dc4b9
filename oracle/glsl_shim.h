/*
 * GLSL-in-C++ shim: just enough of the GLSL language (vector/matrix types, swizzles, built-in
 * functions, integer/float conversions, single-invocation subgroup operations) to compile the
 * reference's own setup, binning, row-span, shading and reduction functions
 * (data/shaders/quad_setup.glsl, bin_counter.glsl, raster_low.glsl, shared/*.glsl) as plain C++
 * on the CPU.
 *
 * TEST INFRASTRUCTURE ONLY: used by oracle/ref_build.py to build oracle/_ref, which pins the
 * oracle's setup records to the reference's source. Nothing in lucid_gb300/ uses it.
 *
 * Float semantics follow the numerics contract shared by the oracle and the CUDA path: every
 * operation rounds to FP32 (built with -ffp-contract=off), dot products and matrix-vector
 * products accumulate left to right ((a.x*b.x + a.y*b.y) + a.z*b.z; ((c0*x + c1*y) + c2*z) + c3*w),
 * length(v) = sqrt(dot(v, v)), int()/uint() of a float truncate. The GLSL source fixes the
 * expressions; these orders are the ones the shader compilers' straightforward lowering gives.
 */
#ifndef LUCID_GLSL_SHIM_H
#define LUCID_GLSL_SHIM_H

#include <cmath>
#include <cstdint>
#include <cstring>

namespace glsl {

typedef uint32_t uint;

template <class T, int N> struct vecN;

// Swizzle of components (i0, i1[, i2]) of a vector: reads as a vector, writes back through
// compound assignment.
template <class T, int N, int M> struct Swz {
	T* base;
	int idx[M];
	operator vecN<T, M>() const;
	template <class U> Swz& operator*=(U s) {
		for(int k = 0; k < M; k++)
			base[idx[k]] = base[idx[k]] * T(s);
		return *this;
	}
	Swz& operator=(const vecN<T, M>& v);
};

template <class T, int N> struct vecN;

template <class T> struct vecN<T, 2> {
	T x, y;
	vecN() : x(0), y(0) {}
	explicit vecN(T s) : x(s), y(s) {}
	vecN(T a, T b) : x(a), y(b) {}
	template <class U> explicit vecN(const vecN<U, 2>& o) : x(T(o.x)), y(T(o.y)) {}
	T& operator[](int i) { return (&x)[i]; }
	T operator[](int i) const { return (&x)[i]; }
};

template <class T> struct vecN<T, 3> {
	T x, y, z;
	vecN() : x(0), y(0), z(0) {}
	explicit vecN(T s) : x(s), y(s), z(s) {}
	vecN(T a, T b, T c) : x(a), y(b), z(c) {}
	template <class U> explicit vecN(const vecN<U, 3>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
	T& operator[](int i) { return (&x)[i]; }
	T operator[](int i) const { return (&x)[i]; }
	vecN<T, 2> xy() const { return vecN<T, 2>(x, y); }
};

template <class T> struct vecN<T, 4> {
	T x, y, z, w;
	vecN() : x(0), y(0), z(0), w(0) {}
	explicit vecN(T s) : x(s), y(s), z(s), w(s) {}
	vecN(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
	vecN(const vecN<T, 3>& v, T d) : x(v.x), y(v.y), z(v.z), w(d) {}
	template <class U> vecN(const vecN<U, 2>& a, const vecN<U, 2>& b) : x(T(a.x)), y(T(a.y)), z(T(b.x)), w(T(b.y)) {}
	template <class U> explicit vecN(const vecN<U, 4>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)), w(T(o.w)) {}
	T& operator[](int i) { return (&x)[i]; }
	T operator[](int i) const { return (&x)[i]; }
	vecN<T, 2> xy() const { return vecN<T, 2>(x, y); }
	vecN<T, 2> zw() const { return vecN<T, 2>(z, w); }
	Swz<T, 4, 3> xyz() { return Swz<T, 4, 3>{&x, {0, 1, 2}}; }
	vecN<T, 3> xyz() const { return vecN<T, 3>(x, y, z); }
	Swz<T, 4, 3> rgb() { return Swz<T, 4, 3>{&x, {0, 1, 2}}; }
	vecN<T, 3> rgb() const { return vecN<T, 3>(x, y, z); }
	vecN<T, 3> xzw() const { return vecN<T, 3>(x, z, w); }
};

template <class T, int N, int M> Swz<T, N, M>::operator vecN<T, M>() const {
	vecN<T, M> r;
	for(int k = 0; k < M; k++)
		r[k] = base[idx[k]];
	return r;
}
template <class T, int N, int M> Swz<T, N, M>& Swz<T, N, M>::operator=(const vecN<T, M>& v) {
	for(int k = 0; k < M; k++)
		base[idx[k]] = v[k];
	return *this;
}

typedef vecN<float, 2> vec2;
typedef vecN<float, 3> vec3;
typedef vecN<float, 4> vec4;
typedef vecN<int, 2> ivec2;
typedef vecN<int, 4> ivec4;
typedef vecN<uint, 2> uvec2;
typedef vecN<uint, 3> uvec3;
typedef vecN<uint, 4> uvec4;
typedef vecN<bool, 3> bvec3;

// componentwise operators (evaluated component by component, each rounding to T)
#define LUCID_SHIM_BINOP(OP)                                                                          \
	template <class T, int N> vecN<T, N> operator OP(const vecN<T, N>& a, const vecN<T, N>& b) {       \
		vecN<T, N> r;                                                                                  \
		for(int i = 0; i < N; i++)                                                                     \
			r[i] = a[i] OP b[i];                                                                       \
		return r;                                                                                      \
	}                                                                                                  \
	template <class T, int N, class U> vecN<T, N> operator OP(const vecN<T, N>& a, U s) {             \
		vecN<T, N> r;                                                                                  \
		for(int i = 0; i < N; i++)                                                                     \
			r[i] = a[i] OP T(s);                                                                       \
		return r;                                                                                      \
	}                                                                                                  \
	template <class T, int N> vecN<T, N>& operator OP##=(vecN<T, N>& a, const vecN<T, N>& b) {         \
		return a = a OP b;                                                                             \
	}                                                                                                  \
	template <class T, int N, class U> vecN<T, N>& operator OP##=(vecN<T, N>& a, U s) { return a = a OP s; }
LUCID_SHIM_BINOP(+)
LUCID_SHIM_BINOP(-)
LUCID_SHIM_BINOP(*)
LUCID_SHIM_BINOP(/)
#undef LUCID_SHIM_BINOP

// scalar on the left: componentwise s OP v[i]
#define LUCID_SHIM_SCALAR_LEFT(OP)                                                                    \
	template <class T, int N> vecN<T, N> operator OP(T s, const vecN<T, N>& a) {                       \
		vecN<T, N> r;                                                                                  \
		for(int i = 0; i < N; i++)                                                                     \
			r[i] = s OP a[i];                                                                          \
		return r;                                                                                      \
	}
LUCID_SHIM_SCALAR_LEFT(+)
LUCID_SHIM_SCALAR_LEFT(-)
LUCID_SHIM_SCALAR_LEFT(*)
#undef LUCID_SHIM_SCALAR_LEFT

// a swizzle in an expression reads as its vector
template <class T, int N, int M> vecN<T, M> swzValue(const Swz<T, N, M>& s) { return vecN<T, M>(s); }
template <class T, int N, int M> vecN<T, M> operator-(const Swz<T, N, M>& s) { return -swzValue(s); }
template <class T, int N, int M, class U> auto operator*(const Swz<T, N, M>& a, const U& b) { return swzValue(a) * b; }
template <class T, int N, int M> vecN<T, M> operator*(T b, const Swz<T, N, M>& a) { return b * swzValue(a); }

template <class T, int N> vecN<T, N> operator-(const vecN<T, N>& a) {
	vecN<T, N> r;
	for(int i = 0; i < N; i++)
		r[i] = -a[i];
	return r;
}
template <class T, int N> vecN<T, N> operator>>(const vecN<T, N>& a, int s) {
	vecN<T, N> r;
	for(int i = 0; i < N; i++)
		r[i] = a[i] >> s;
	return r;
}
// GLSL == on vectors: all components equal
template <class T, int N> bool operator==(const vecN<T, N>& a, const vecN<T, N>& b) {
	for(int i = 0; i < N; i++)
		if(!(a[i] == b[i]))
			return false;
	return true;
}

struct mat4 {
	vec4 col[4];
};
// ((c0 * x + c1 * y) + c2 * z) + c3 * w, per row
inline vec4 operator*(const mat4& m, const vec4& v) {
	vec4 r;
	for(int i = 0; i < 4; i++)
		r[i] = ((m.col[0][i] * v.x + m.col[1][i] * v.y) + m.col[2][i] * v.z) + m.col[3][i] * v.w;
	return r;
}

inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline vec3 cross(const vec3& a, const vec3& b) {
	return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float length(const vec3& v) { return std::sqrt(dot(v, v)); }

// GLSL min/max/clamp: NaN handling as fminf/fmaxf (the non-NaN operand)
inline float min(float a, float b) { return std::fmin(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
template <int N> vecN<float, N> min(const vecN<float, N>& a, const vecN<float, N>& b) {
	vecN<float, N> r;
	for(int i = 0; i < N; i++)
		r[i] = std::fmin(a[i], b[i]);
	return r;
}
template <int N> vecN<float, N> max(const vecN<float, N>& a, const vecN<float, N>& b) {
	vecN<float, N> r;
	for(int i = 0; i < N; i++)
		r[i] = std::fmax(a[i], b[i]);
	return r;
}
template <int N> vecN<float, N> clamp(const vecN<float, N>& v, const vecN<float, N>& lo, const vecN<float, N>& hi) {
	return min(max(v, lo), hi);
}
// clamp(v, 0.0, 1.0) of a float vector (SATURATE): min(max(v, lo), hi) per component
template <int N> vecN<float, N> clamp(const vecN<float, N>& v, double lo, double hi) {
	return min(max(v, vecN<float, N>(float(lo))), vecN<float, N>(float(hi)));
}
template <int N> vecN<float, N> fract(const vecN<float, N>& v) {
	vecN<float, N> r;
	for(int i = 0; i < N; i++)
		r[i] = v[i] - std::floor(v[i]);
	return r;
}
inline float min(float a, int b) { return std::fmin(a, float(b)); }
inline float max(float a, int b) { return std::fmax(a, float(b)); }
inline int clamp(int v, int lo, int hi) { return min(max(v, lo), hi); }
inline float ceil(float x) { return std::ceil(x); }
inline float floor(float x) { return std::floor(x); }

inline uint floatBitsToUint(float f) {
	uint u;
	std::memcpy(&u, &f, 4);
	return u;
}
template <int N> vecN<uint, N> floatBitsToUint(const vecN<float, N>& v) {
	vecN<uint, N> r;
	for(int i = 0; i < N; i++)
		r[i] = floatBitsToUint(v[i]);
	return r;
}
inline float uintBitsToFloat(uint u) {
	float f;
	std::memcpy(&f, &u, 4);
	return f;
}
inline vec3 uintBitsToFloat(const uvec3& v) {
	return vec3(uintBitsToFloat(v.x), uintBitsToFloat(v.y), uintBitsToFloat(v.z));
}
inline vec2 uintBitsToFloat(const uvec2& v) { return vec2(uintBitsToFloat(v.x), uintBitsToFloat(v.y)); }

// GLSL pow is implementation-defined; the harness points this at the pow that the oracle and
// the CUDA path share (the oracle's refPow)
extern float (*g_pow)(float, float);
inline float pow(float x, float y) { return g_pow(x, y); }

// integer bit functions
inline int bitCount(uint v) { return __builtin_popcount(v); }
inline int findLSB(uint v) { return v ? __builtin_ctz(v) : -1; }

// subgroup operations of one invocation running alone: a vote is its own predicate, a shuffle
// returns its own value
inline bool subgroupAny(bool b) { return b; }
inline bool subgroupAll(bool b) { return b; }
template <class T> T subgroupShuffle(const T& v, int) { return v; }

// textures are outside the pinned functions: the stub marks a call, and the tests use scenes
// without textures
struct sampler2D {
	int unused;
};
extern int g_texture_calls;
inline vec4 textureGrad(const sampler2D&, const vec2&, const vec2&, const vec2&) {
	g_texture_calls++;
	return vec4(NAN);
}

// int() / uint() conversions. Of a float: truncation toward zero, saturating at the type's
// limits, NaN to 0 (GLSL leaves out-of-range values undefined; this is what the GPU's conversion
// instruction does, and what the oracle emulates). Of an integer: the value.
inline int toInt(float x) {
	if(x != x)
		return 0;
	if(x >= 2147483648.0f)
		return 2147483647;
	if(x <= -2147483648.0f)
		return int(0x80000000u);
	return int(x);
}
inline int toInt(int x) { return x; }
inline int toInt(uint x) { return int(x); }
inline uint toUint(float x) {
	if(x != x || x <= 0.0f)
		return 0u;
	if(x >= 4294967296.0f)
		return 0xffffffffu;
	return uint(x);
}
inline uint toUint(int x) { return uint(x); }
inline uint toUint(uint x) { return x; }
inline uvec4 toUvec4(const vec4& v) { return uvec4(toUint(v.x), toUint(v.y), toUint(v.z), toUint(v.w)); }

// atomicAdd on a variable of a sequentially emulated invocation: returns the old value
template <class T, class U> T atomicAdd(T& x, U v) {
	T old = x;
	x = T(x + v);
	return old;
}

} // namespace glsl

#endif
