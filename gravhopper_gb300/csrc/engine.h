// Internal C++ interface between the C-ABI layer (capi.cu) and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gh {

// Direct-sum acceleration in code units (G=1, kpc, Msun).  tpos == nullptr means
// targets are the sources (self term skipped, reference direct_summation).
int direct_force(const double* pos, const double* mass, int64_t np, const double* tpos, int64_t nt,
                 double eps, int precision, double* acc, cudaStream_t st);

// Selects the tile shape of the mixed direct kernel (index into kMixedShapes).
int set_mixed_shape(int shape);
// Autotuned shape rules (gh_direct_tune) and the shape a size would get.
int tune_rule(int64_t n_min, int fused_step, int shape);
int shape_for(int64_t n, int fused_step);
int set_f64_form(int form);

// `nsteps` leapfrog steps with the direct force, one fused launch per step.
int direct_run(double* x, double* v, const double* mass, int64_t np, int64_t nsteps, double dt,
               double eps, int precision, double* hist_x, double* hist_v, int64_t stride,
               cudaStream_t st);

// First half-drift of a run into an FP64 (N,3) array: xh = x + ((0.5*v)*dt)*F.
int drift_prepare_f64(const double* x, const double* v, int64_t n, double dt, double* xh, cudaStream_t st);

// Barnes-Hut acceleration in code units (tpos == nullptr: targets are the sources).
int tree_force(const double* pos, const double* mass, int64_t np, const double* tpos, int64_t nt,
               double eps, double theta, int precision, double* acc, cudaStream_t st);

// `nsteps` leapfrog steps with the tree force (rebuilt every step).
int tree_run(double* x, double* v, const double* mass, int64_t np, int64_t nsteps, double dt,
             double eps, double theta, int precision, double* hist_x, double* hist_v, int64_t stride,
             cudaStream_t st);

// VJP of the direct-sum acceleration (adjoint.cu): cotangent lam (N,3) -> gradients
// with respect to positions (N,3) and masses (N, may be null).
int direct_vjp(const double* pos, const double* mass, int64_t n, double eps, const double* lam, int precision,
               double* gpos, double* gmass, cudaStream_t st);

// Reverse pass of nsteps direct-sum DKD steps starting from (x0, v0): recomputes the
// states, then updates the cotangents (xbar, vbar) in place and adds to mbar.
int dkd_backward(const double* x0, const double* v0, const double* mass, int64_t n, int64_t nsteps, double dt,
                 double eps, int precision, double* xbar, double* vbar, double* mbar, cudaStream_t st);
int dkd_backward_chain(const double* cx, const double* cv, const int64_t* seg, int64_t nseg, const double* mass,
                       int64_t n, double dt, double eps, int precision, double* xbar, double* vbar, double* mbar,
                       cudaStream_t st);

// Per-particle softened potential phi_k = -sum_{j != k} m_j / sqrt(r^2 + eps^2) (G=1).
int potential(const double* pos, const double* mass, int64_t n, double eps, double* phi, cudaStream_t st);

// Batched leapfrog of nsys independent systems (mixed precision), see ensemble.cu.
int ensemble_run(double* x, double* v, const double* mass, const int64_t* h_off, int64_t nsys, const double* h_eps,
                 const double* h_dt, int64_t nsteps, int config, int use_graph, cudaStream_t st);
int ensemble_num_configs();

}  // namespace gh
