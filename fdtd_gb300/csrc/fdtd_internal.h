// fdtd_internal.h -- declarations shared by the library's translation units.
#pragma once

#include "../../include/fdtd_gb300.h"

#include <cstddef>
#include <cstdint>
#include <functional>
#include <string>

namespace fdtd {

// Host thread pool helpers (host_io.cpp).
int host_threads(int requested);
void parallel_for(int n, int nthreads, const std::function<void(int)> &fn);

// Mur slab value for one material (host_io.cpp).
float mur_rp_value(const FdtdParams *p, float sigma, float eps_s, float eps_i, float tau, bool imaginary);

// Text snapshot helpers (host_io.cpp).
int write_plane_text(const std::string &path, const float *plane, int nx, int ny);
std::string snapshot_name(const char *dir, int field, int iteration, int z);
// Binary snapshot file of nplanes planes from z0, and a raw float writer.
std::string snapshot_name_f32(const char *dir, int field, int iteration, int z0, int nplanes);
int write_floats(const std::string &path, const float *data, size_t count);

// cudaGetErrorString for codes below FDTD_ERR_INVALID (cuda_util.cu).
const char *cuda_error_string(int code);

// Debye coefficients of one material class, computed on the host exactly as
// updateEField computes them per cell (fdtd_calculations.cu:141-144): a, b, c,
// d are double expressions stored as float.  The D terms of the update are
// applied in the difference form
//   k1 D0 - k2 D1 + k3 D2 = two_dt (D0 - D1) + two_tau ((D0 - D1) - (D1 - D2)) + delta D0
// with two_dt = 2 dt, two_tau = 2 tau and delta = 2 (fl(dt + tau) - (dt + tau)),
// which is exact algebra for the reference's k1 = 2 fl(dt + tau),
// k2 = 2 dt + 4 tau, k3 = 2 tau and avoids the cancellation of the three
// large products in single precision.
struct alignas(16) DebyeCoef {
    float a, c, d, two_dt, two_tau, delta, pad0, pad1;
};
static_assert(sizeof(DebyeCoef) == 32, "DebyeCoef is two float4");

DebyeCoef debye_coef(float dt, float eps0, float sigma, float eps_s, float eps_i, float tau, int scheme);

}  // namespace fdtd
