// ORACLE — test infrastructure only. Not part of the shipped library.
//
// CPU restatement of OSL's forward-mode derivative type Dual2<T> and the
// small vector type it is used with. Operation order (which operand is
// multiplied first, which partial is added first) follows
// src/include/OSL/dual.h:403-620 so that the float results of every noise
// and arithmetic op computed on top of it are the reference's, operation for
// operation. Compile with -ffp-contract=off: the reference's non-FMA batched
// targets build the shadeop library with contraction disabled
// (src/liboslexec/CMakeLists.txt:392-399), and that is the order this oracle
// pins.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace oracle {

struct V3 {
    float x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(float a) : x(a), y(a), z(a) {}
    V3(float a, float b, float c) : x(a), y(b), z(c) {}
    float& operator[](int i) { return (&x)[i]; }
    float operator[](int i) const { return (&x)[i]; }
};
inline V3 operator+(const V3& a, const V3& b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(const V3& a, const V3& b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator-(const V3& a) { return V3(-a.x, -a.y, -a.z); }
inline V3 operator*(const V3& a, const V3& b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline V3 operator*(const V3& a, float b) { return V3(a.x * b, a.y * b, a.z * b); }
inline V3 operator*(float b, const V3& a) { return V3(b * a.x, b * a.y, b * a.z); }
inline V3 operator/(const V3& a, const V3& b) { return V3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline V3 operator/(const V3& a, float b) { return V3(a.x / b, a.y / b, a.z / b); }

// Dual2<T>: value plus x and y partials (dual.h:228, Dual<T,2>).
template <class T> struct Dual2 {
    T v, dx, dy;
    Dual2() : v(T(0.0f)), dx(T(0.0f)), dy(T(0.0f)) {}
    Dual2(const T& a) : v(a), dx(T(0.0f)), dy(T(0.0f)) {}
    Dual2(const T& a, const T& b, const T& c) : v(a), dx(b), dy(c) {}
    const T& val() const { return v; }
};
typedef Dual2<float> DF;
typedef Dual2<V3> DV;

// dual.h:403 a+b, :415 a+scalar, :424 scalar+a
template <class T> inline Dual2<T> operator+(const Dual2<T>& a, const Dual2<T>& b) {
    return Dual2<T>(a.v + b.v, a.dx + b.dx, a.dy + b.dy);
}
template <class T> inline Dual2<T> operator+(const Dual2<T>& a, const T& b) {
    return Dual2<T>(a.v + b, a.dx, a.dy);
}
template <class T> inline Dual2<T> operator+(const T& a, const Dual2<T>& b) {
    return Dual2<T>(b.v + a, b.dx, b.dy);
}
// dual.h:453 a-b, :464 a-scalar, :473 scalar-a, :506 unary minus
template <class T> inline Dual2<T> operator-(const Dual2<T>& a, const Dual2<T>& b) {
    return Dual2<T>(a.v - b.v, a.dx - b.dx, a.dy - b.dy);
}
template <class T> inline Dual2<T> operator-(const Dual2<T>& a, const T& b) {
    return Dual2<T>(a.v - b, a.dx, a.dy);
}
template <class T> inline Dual2<T> operator-(const T& a, const Dual2<T>& b) {
    return Dual2<T>(a - b.v, -b.dx, -b.dy);
}
template <class T> inline Dual2<T> operator-(const Dual2<T>& a) {
    return Dual2<T>(-a.v, -a.dx, -a.dy);
}
// dual.h:518-532: chain rule, partial = a.val*b.partial + a.partial*b.val
inline DF operator*(const DF& a, const DF& b) {
    return DF(a.v * b.v, a.v * b.dx + a.dx * b.v, a.v * b.dy + a.dy * b.v);
}
inline DV operator*(const DV& a, const DF& b) {
    return DV(a.v * b.v, a.v * b.dx + a.dx * b.v, a.v * b.dy + a.dy * b.v);
}
inline DV operator*(const DF& a, const DV& b) {
    return DV(a.v * b.v, a.v * b.dx + a.dx * b.v, a.v * b.dy + a.dy * b.v);
}
inline DV operator*(const DV& a, const DV& b) {
    return DV(a.v * b.v, a.v * b.dx + a.dx * b.v, a.v * b.dy + a.dy * b.v);
}
// dual.h:534-572: dual times a non-dual scalar multiplies every element
template <class T, class S> inline Dual2<T> operator*(const Dual2<T>& a, const S& b) {
    return Dual2<T>(a.v * b, a.dx * b, a.dy * b);
}
template <class T, class S> inline Dual2<T> operator*(const S& b, const Dual2<T>& a) {
    return a * b;
}
// dual.h:575-589
inline DF operator/(const DF& a, const DF& b) {
    float binv = 1.0f / b.v;
    float ab = a.v / b.v;
    return DF(ab, binv * (a.dx - ab * b.dx), binv * (a.dy - ab * b.dy));
}
// dual.h:592-605
inline DF operator/(const DF& a, float b) {
    float binv = 1.0f / b;
    float ab = a.v / b;
    return DF(ab, binv * a.dx, binv * a.dy);
}
// dual.h:608-620
inline DF operator/(float a, const DF& b) {
    float binv = 1.0f / b.v;
    float ab = a / b.v;
    return DF(ab, binv * (-ab * b.dx), binv * (-ab * b.dy));
}

// Channel accessors used by the Vec3 <-> float decomposition in the noise
// wrappers (oslnoise.h:2364-2366 builds Dual2<float> px from p.val().x ...).
inline DF comp(const DV& a, int c) { return DF(a.v[c], a.dx[c], a.dy[c]); }
inline void setcomp(DV& a, int c, const DF& f) { a.v[c] = f.v; a.dx[c] = f.dx; a.dy[c] = f.dy; }

inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float bitsf(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

}  // namespace oracle
