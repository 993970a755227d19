// The drift-kick-drift step split in two launches, for runs whose acceleration has a
// part computed outside this library (external forces, gravhopper.py:462-473): the
// first drift, then the caller's N-body force and external acceleration, then the
// kick and the second drift.  Simulation.perform_timestep (gravhopper.py:405-416) in
// the same operations and order as the fused step, with the external acceleration
// added to the N-body one as calculate_acceleration does (nbody + extra, :459):
//   xh = x + ((0.5*v)*dt)*F
//   v' = v + ((a*ACC) + ext)*dt
//   x' = xh + ((0.5*v')*dt)*F
// Elementwise and HBM-bound: 48 B read and 24 B written per particle for the drift,
// 96 B read and 48 B written for the kick and drift.
#include "direct.cuh"

namespace gh {

constexpr int LF_THREADS = 256;

__global__ void __launch_bounds__(LF_THREADS)
    lf_drift_kernel(const double* __restrict__ x, const double* __restrict__ v, int64_t n3, double dt,
                    double* __restrict__ xh) {
  for (int64_t k = (int64_t)blockIdx.x * LF_THREADS + threadIdx.x; k < n3; k += (int64_t)gridDim.x * LF_THREADS)
    xh[k] = drift_half(x[k], v[k], dt);
}

__global__ void __launch_bounds__(LF_THREADS)
    lf_kick_drift_kernel(const double* __restrict__ xh, double* __restrict__ v, const double* __restrict__ acc,
                         const double* __restrict__ ext, int64_t n3, double dt, double* __restrict__ xout) {
  for (int64_t k = (int64_t)blockIdx.x * LF_THREADS + threadIdx.x; k < n3; k += (int64_t)gridDim.x * LF_THREADS) {
    double a = acc ? dmul(acc[k], GH_ACCEL_UNIT) : 0.0;  // no N-body force (np <= 1): zeros
    if (ext) a = dadd(a, ext[k]);
    const double v1 = dadd(v[k], dmul(a, dt));
    v[k] = v1;
    xout[k] = drift_half(xh[k], v1, dt);
  }
}

static unsigned lf_grid(int64_t n3) {
  DeviceInfo di;
  const int64_t cap = device_info(&di) == GH_OK ? (int64_t)di.num_sms * 8 : 1216;
  const int64_t need = (n3 + LF_THREADS - 1) / LF_THREADS;
  return (unsigned)(need < cap ? need : cap);
}

}  // namespace gh

using namespace gh;

extern "C" int gh_dkd_drift(const double* pos, const double* vel, int64_t np, double dt, double* pos_half,
                            void* stream) {
  clear_error();
  if (np < 0) return set_error(GH_ERR_ARG, "negative np");
  if (np == 0) return GH_OK;
  if (!pos || !vel || !pos_half) return set_error(GH_ERR_ARG, "null buffer");
  const int64_t n3 = 3 * np;
  lf_drift_kernel<<<lf_grid(n3), LF_THREADS, 0, (cudaStream_t)stream>>>(pos, vel, n3, dt, pos_half);
  GH_LAUNCH_CHECK();
  return GH_OK;
}

extern "C" int gh_dkd_kick_drift(const double* pos_half, double* vel, const double* acc, const double* acc_ext,
                                 int64_t np, double dt, double* pos_out, void* stream) {
  clear_error();
  if (np < 0) return set_error(GH_ERR_ARG, "negative np");
  if (np == 0) return GH_OK;
  if (!pos_half || !vel || !pos_out) return set_error(GH_ERR_ARG, "null buffer");
  const int64_t n3 = 3 * np;
  lf_kick_drift_kernel<<<lf_grid(n3), LF_THREADS, 0, (cudaStream_t)stream>>>(pos_half, vel, acc, acc_ext, n3, dt,
                                                                             pos_out);
  GH_LAUNCH_CHECK();
  return GH_OK;
}
