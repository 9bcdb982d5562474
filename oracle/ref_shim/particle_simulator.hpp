// particle_simulator.hpp — minimal single-rank stand-in for the FDPS types
// that the reference's functor headers (hdr_run, hdr_dimension, hdr_kernel,
// hdr_sph, hdr_density, hdr_hydro, hdr_gravity) use.  TEST INFRASTRUCTURE:
// it exists only so that oracle/ref_bridge.cpp can compile those headers from
// the reference tree as the parity oracle.  It holds no FDPS code: only the
// scalar typedefs, a 3-vector, a symmetric 3x3 matrix, an orthotope and a
// one-rank Comm.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <iostream>

namespace ParticleSimulator {

typedef float F32;
typedef double F64;
typedef int32_t S32;
typedef int64_t S64;
typedef uint64_t U64;

template <class T>
struct Vector3 {
    T x, y, z;
    Vector3() : x(0), y(0), z(0) {}
    Vector3(T s) : x(s), y(s), z(s) {}
    Vector3(T a, T b, T c) : x(a), y(b), z(c) {}
    template <class U>
    Vector3(const Vector3<U> &o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}

    T &operator[](int k) { return k == 0 ? x : (k == 1 ? y : z); }
    const T &operator[](int k) const { return k == 0 ? x : (k == 1 ? y : z); }

    Vector3 operator+(const Vector3 &o) const { return Vector3(x + o.x, y + o.y, z + o.z); }
    Vector3 operator-(const Vector3 &o) const { return Vector3(x - o.x, y - o.y, z - o.z); }
    Vector3 operator-() const { return Vector3(-x, -y, -z); }
    Vector3 operator*(T s) const { return Vector3(x * s, y * s, z * s); }
    // FDPS convention: vector * vector is the dot product, ^ the cross product.
    T operator*(const Vector3 &o) const { return x * o.x + y * o.y + z * o.z; }
    Vector3 operator^(const Vector3 &o) const {
        return Vector3(y * o.z - z * o.y, z * o.x - x * o.z, x * o.y - y * o.x);
    }
    Vector3 &operator+=(const Vector3 &o) { x += o.x; y += o.y; z += o.z; return *this; }
    Vector3 &operator-=(const Vector3 &o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    Vector3 &operator*=(T s) { x *= s; y *= s; z *= s; return *this; }
};

template <class T>
inline Vector3<T> operator*(T s, const Vector3<T> &v) { return v * s; }

template <class T>
inline std::ostream &operator<<(std::ostream &os, const Vector3<T> &v) {
    return os << v.x << " " << v.y << " " << v.z;
}

typedef Vector3<F32> F32vec;
typedef Vector3<F64> F64vec;

struct F64mat {
    F64 xx, yy, zz, xy, xz, yz;
    F64mat() : xx(0), yy(0), zz(0), xy(0), xz(0), yz(0) {}
    F64mat(F64 s) : xx(s), yy(s), zz(s), xy(s), xz(s), yz(s) {}
};

struct F64ort {
    F64vec low_, high_;
};

namespace Comm {
inline S32 getRank() { return 0; }
inline S32 getNumberOfProc() { return 1; }
template <class T> inline T getSum(const T &v) { return v; }
template <class T> inline T getMinValue(const T &v) { return v; }
template <class T> inline T getMaxValue(const T &v) { return v; }
inline bool synchronizeConditionalBranchOR(bool v) { return v; }
inline void barrier() {}
}  // namespace Comm

inline void Abort(int = -1) { std::abort(); }

}  // namespace ParticleSimulator

namespace PS = ParticleSimulator;
