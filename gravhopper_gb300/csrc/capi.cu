// extern "C" entry points: host-buffer drop-ins for gravhopper._jbgrav and the
// device-pointer, stream-ordered calls.
#include <mutex>

#include "direct.cuh"
#include "engine.h"
#include "gh_common.cuh"

namespace gh {

// Staging buffers and a private stream for the host-buffer entry points.
struct HostStage {
  Buffer pos, mass, tpos, out;
  cudaStream_t stream = nullptr;
};
static HostStage g_stage[64];
static std::mutex g_stage_mu;

static int stage_for_device(HostStage** out) {
  DeviceInfo di;
  GH_TRY(device_info(&di));
  HostStage& s = g_stage[di.device];
  if (!s.stream) GH_CUDA_TRY(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking));
  *out = &s;
  return GH_OK;
}

enum HostKind { HK_DIRECT = 0, HK_TREE = 1 };

// Shared body of the host-buffer calls: copy in, compute, copy out, synchronise.
static int host_call(HostKind kind, const double* pos, const double* mass, int64_t np,
                     const double* tpos, int64_t nt, double eps, int precision, double theta,
                     double* out) {
  clear_error();
  if (np < 0 || nt < 0)
    return set_error(GH_ERR_ARG, "negative particle count (np=%lld, nf=%lld)", (long long)np,
                     (long long)nt);
  const bool self = (tpos == nullptr);
  const int64_t n_out = self ? np : nt;
  if (n_out == 0) return GH_OK;
  if (!out || (np > 0 && (!pos || !mass)))
    return set_error(GH_ERR_ARG, "null host buffer");
  Trace tr(kind == HK_DIRECT ? "gh host direct sum" : "gh host tree force");
  std::lock_guard<std::mutex> lk(g_stage_mu);
  HostStage* s = nullptr;
  GH_TRY(stage_for_device(&s));
  const size_t pb = (size_t)np * 3 * sizeof(double);
  const size_t tb = (size_t)nt * 3 * sizeof(double);
  const size_t ob = (size_t)n_out * 3 * sizeof(double);
  GH_TRY(ensure(s->pos, pb ? pb : 8));
  GH_TRY(ensure(s->mass, np ? (size_t)np * sizeof(double) : 8));
  GH_TRY(ensure(s->out, ob));
  if (np) {
    GH_CUDA_TRY(cudaMemcpyAsync(s->pos.ptr, pos, pb, cudaMemcpyHostToDevice, s->stream));
    GH_CUDA_TRY(cudaMemcpyAsync(s->mass.ptr, mass, (size_t)np * sizeof(double),
                                cudaMemcpyHostToDevice, s->stream));
  }
  const double* dt = nullptr;
  if (!self) {
    GH_TRY(ensure(s->tpos, tb));
    GH_CUDA_TRY(cudaMemcpyAsync(s->tpos.ptr, tpos, tb, cudaMemcpyHostToDevice, s->stream));
    dt = (const double*)s->tpos.ptr;
  }
  int rc;
  if (kind == HK_DIRECT)
    rc = direct_force((const double*)s->pos.ptr, (const double*)s->mass.ptr, np, dt, nt, eps,
                      precision, (double*)s->out.ptr, s->stream);
  else
    rc = tree_force((const double*)s->pos.ptr, (const double*)s->mass.ptr, np, dt, nt, eps, theta, precision,
                    (double*)s->out.ptr, s->stream);
  if (rc != GH_OK) {
    cudaStreamSynchronize(s->stream);
    return rc;
  }
  GH_CUDA_TRY(cudaMemcpyAsync(out, s->out.ptr, ob, cudaMemcpyDeviceToHost, s->stream));
  GH_CUDA_TRY(cudaStreamSynchronize(s->stream));
  return GH_OK;
}

}  // namespace gh

using namespace gh;

extern "C" {

int gh_direct_summation(const double* pos, const double* mass, int64_t np, double eps,
                        double* out) {
  return host_call(HK_DIRECT, pos, mass, np, nullptr, 0, eps, GH_PREC_FP64, 0.0, out);
}

int gh_direct_summation_position(const double* pos, const double* mass, int64_t np,
                                 const double* force_pos, int64_t nf, double eps, double* out) {
  if (!force_pos && nf > 0) return set_error(GH_ERR_ARG, "force_pos is NULL");
  if (nf == 0) return GH_OK;
  return host_call(HK_DIRECT, pos, mass, np, force_pos, nf, eps, GH_PREC_FP64, 0.0, out);
}

int gh_tree_force(const double* pos, const double* mass, int64_t np, double eps, double theta,
                  double* out) {
  return host_call(HK_TREE, pos, mass, np, nullptr, 0, eps, GH_PREC_FP64, theta, out);
}

int gh_tree_force_position(const double* pos, const double* mass, int64_t np, const double* force_pos,
                           int64_t nf, double eps, double theta, double* out) {
  if (!force_pos && nf > 0) return set_error(GH_ERR_ARG, "force_pos is NULL");
  if (nf == 0) return GH_OK;
  return host_call(HK_TREE, pos, mass, np, force_pos, nf, eps, GH_PREC_FP64, theta, out);
}

int gh_tree_dev(const double* pos, const double* mass, int64_t np, const double* force_pos, int64_t nf,
                double eps, double theta, int precision, double* acc, void* stream) {
  clear_error();
  Trace tr("gh_tree_dev");
  return tree_force(pos, mass, np, force_pos, nf, eps, theta, precision, acc, (cudaStream_t)stream);
}

int gh_direct_host(const double* pos, const double* mass, int64_t np, const double* force_pos,
                   int64_t nf, double eps, int precision, double* out) {
  return host_call(HK_DIRECT, pos, mass, np, force_pos, nf, eps, precision, 0.0, out);
}

int gh_direct_dev(const double* pos, const double* mass, int64_t np, const double* force_pos,
                  int64_t nf, double eps, int precision, double* acc, void* stream) {
  clear_error();
  Trace tr("gh_direct_dev");
  return direct_force(pos, mass, np, force_pos, nf, eps, precision, acc, (cudaStream_t)stream);
}

int gh_run_dkd(double* pos, double* vel, const double* mass, int64_t np, int64_t nsteps,
               double dt, double eps, int algorithm, int precision, double theta,
               double* hist_pos, double* hist_vel, int64_t hist_stride, void* stream) {
  clear_error();
  Trace tr("gh_run_dkd");
  if (np < 0 || nsteps < 0) return set_error(GH_ERR_ARG, "negative np or nsteps");
  if (algorithm != GH_ALGO_DIRECT && algorithm != GH_ALGO_TREE)
    return set_error(GH_ERR_ARG, "unknown algorithm %d", algorithm);
  if (precision != GH_PREC_FP64 && precision != GH_PREC_MIXED)
    return set_error(GH_ERR_ARG, "unknown precision %d", precision);
  if (!(eps >= 0.0)) return set_error(GH_ERR_ARG, "eps must be >= 0");
  if ((hist_pos == nullptr) != (hist_vel == nullptr))
    return set_error(GH_ERR_ARG, "hist_pos and hist_vel must both be set or both be NULL");
  if (hist_pos && hist_stride < 1) return set_error(GH_ERR_ARG, "hist_stride must be >= 1");
  if (np == 0 || nsteps == 0) return GH_OK;
  if (!pos || !vel || !mass) return set_error(GH_ERR_ARG, "null state buffer");
  cudaStream_t st = (cudaStream_t)stream;
  if (algorithm == GH_ALGO_DIRECT)
    return direct_run(pos, vel, mass, np, nsteps, dt, eps, precision, hist_pos, hist_vel,
                      hist_stride, st);
  return tree_run(pos, vel, mass, np, nsteps, dt, eps, theta, precision, hist_pos, hist_vel, hist_stride, st);
}

int gh_ensemble_run(double* pos, double* vel, const double* mass, const int64_t* offsets, int64_t nsys,
                    const double* eps, const double* dt, int64_t nsteps, int tile_config, int use_graph,
                    void* stream) {
  clear_error();
  return ensemble_run(pos, vel, mass, offsets, nsys, eps, dt, nsteps, tile_config, use_graph,
                      (cudaStream_t)stream);
}

int gh_ensemble_num_configs(void) { return ensemble_num_configs(); }

int gh_direct_vjp_dev(const double* pos, const double* mass, int64_t np, double eps, const double* cot,
                      int precision, double* grad_pos, double* grad_mass, void* stream) {
  clear_error();
  return direct_vjp(pos, mass, np, eps, cot, precision, grad_pos, grad_mass, (cudaStream_t)stream);
}

int gh_dkd_backward_dev(const double* x0, const double* v0, const double* mass, int64_t np, int64_t nsteps,
                        double dt, double eps, int precision, double* xbar, double* vbar, double* mbar,
                        void* stream) {
  clear_error();
  if (precision != GH_PREC_FP64 && precision != GH_PREC_MIXED)
    return set_error(GH_ERR_ARG, "unknown precision %d", precision);
  if (!(eps >= 0.0)) return set_error(GH_ERR_ARG, "eps must be >= 0");
  return dkd_backward(x0, v0, mass, np, nsteps, dt, eps, precision, xbar, vbar, mbar, (cudaStream_t)stream);
}

int gh_dkd_backward_chain_dev(const double* ckpt_x, const double* ckpt_v, const int64_t* seg_steps, int64_t nseg,
                              const double* mass, int64_t np, double dt, double eps, int precision, double* xbar,
                              double* vbar, double* mbar, void* stream) {
  clear_error();
  if (precision != GH_PREC_FP64 && precision != GH_PREC_MIXED)
    return set_error(GH_ERR_ARG, "unknown precision %d", precision);
  if (!(eps >= 0.0)) return set_error(GH_ERR_ARG, "eps must be >= 0");
  return dkd_backward_chain(ckpt_x, ckpt_v, seg_steps, nseg, mass, np, dt, eps, precision, xbar, vbar, mbar,
                            (cudaStream_t)stream);
}

int gh_potential_dev(const double* pos, const double* mass, int64_t np, double eps, double* phi, void* stream) {
  clear_error();
  return potential(pos, mass, np, eps, phi, (cudaStream_t)stream);
}

int gh_direct_set_shape(int shape) {
  clear_error();
  return set_mixed_shape(shape);
}

int gh_direct_num_shapes(void) { return kNumMixedShapes; }

int gh_direct_tune(int64_t n_min, int fused_step, int shape) {
  clear_error();
  return tune_rule(n_min, fused_step, shape);
}

int gh_direct_shape_for(int64_t n, int fused_step) {
  clear_error();
  if (n < 0 || (fused_step != 0 && fused_step != 1)) return -1;
  return shape_for(n, fused_step);
}

int gh_direct_set_fp64_form(int form) {
  clear_error();
  return set_f64_form(form);
}

}  // extern "C"
