// hgas_shim.hpp — the few FDPS facilities beyond particle_simulator.hpp that
// the reference's hdr_hgas.hpp / hdr_util.hpp name in non-template code
// (vector / scalar, Finalize, thread count, all-to-all on one rank, the
// Mersenne-twister seed call).  TEST INFRASTRUCTURE for oracle/ref_glue.cpp;
// none of these is reached by the functions it binds.
#pragma once

#include <limits>
#include <vector>

#include "particle_simulator.hpp"

namespace ParticleSimulator {
template <class T>
inline Vector3<T> operator/(const Vector3<T> &v, T s) {
    return Vector3<T>(v.x / s, v.y / s, v.z / s);
}
inline void Finalize() {}
namespace Comm {
inline S32 getNumberOfThread() { return 1; }
template <class T>
inline void allToAll(const T *send, int n, T *recv) {
    for (int k = 0; k < n; ++k) recv[k] = send[k];
}
template <class T>
inline void allToAllV(const T *send, const int *n_send, const int *d_send, T *recv, const int *, const int *d_recv) {
    for (int k = 0; k < n_send[0]; ++k) recv[d_recv[0] + k] = send[d_send[0] + k];
}
}  // namespace Comm
namespace MT {
inline void init_genrand(unsigned long) {}
inline double genrand_res53() { return 0.5; }
}  // namespace MT
}  // namespace ParticleSimulator
