// Launchers of the templated kernels, instantiated for float in esm_f32.cu and for double in
// esm_f64.cu (compiled without FMA contraction, the parity build).
#pragma once
#include <cuda_runtime.h>

#include "esm_common.cuh"
#include "esm_linemove.cuh"

namespace esm {
// Load the kernels of the capacity scores now (esm_f64.cu): under lazy module loading a kernel's
// code is placed on the device at its first use, and the score entry point that allocates nothing
// must not be that first use.
cudaError_t preload_score_kernels();
// the fused score pass (esm_kernels_impl.cuh): its step chunks and partial buffer, and its launch
// (instantiated for float and double states in esm_f64.cu, without FMA contraction like the oracle)
template <class S>
cudaError_t launch_scores_fused(const DevModel<double> &M, const S *theta, const S *g, const S *e, const S *z,
                                double *partial, double *sums, cudaStream_t s);
// the FP32 build of the pass (esm_f32.cu): FP32 terms, compensated sums, FP64 balance signs near 0
cudaError_t launch_scores_f32(const DevModel<float> &Mf, const DevModel<double> &Md, double *partial, double *sums,
                              cudaStream_t s);
cudaError_t preload_scores_f32();
template <class real>
cudaError_t launch_rebuild(const DevModel<real> &M, cudaStream_t s);
template <class real>
cudaError_t launch_score_finish(const DevModel<real> &M, const double *k_raw, const double *lo, const double *hi,
                                const double *capex, double gamma_k, double beta_k, int physical, double *sums,
                                double *sk, double *sk_err, double *fk, cudaStream_t s);
template <class real>
cudaError_t launch_follow_disp(const DevModel<real> &M, const int *disp, const double *kold, const double *knew,
                               const double *lo, const double *hi, cudaStream_t s);
template <class real>
cudaError_t launch_kop(const DevModel<real> &M, const double *kold, const double *k1, const double *lo,
                       const double *hi, double kmin, cudaStream_t s);
template <class real>
cudaError_t launch_set_kc(int K, const double *k_raw, const double *lo, const double *hi, const int *u_kind,
                          const int *u_loc, real *kc_d, real *kc_s, real *kc_r, cudaStream_t s);
template <class real>
cudaError_t launch_weather_z(const DevModel<real> &M, const double *phi, const double *mu, const double *season,
                             const double *sig, const double *sig0, const int *moved, const double *theta,
                             const int *regA, const int *regB, const double *xi, uint64_t seed, uint32_t it,
                             int use_theta, cudaStream_t s);
template <class real>
cudaError_t launch_compensate(const DevModel<real> &M, const int *moved, const real *r0, cudaStream_t s);
// the weather features of every replica (esm_kernels_impl.cuh): per-step pass into buf
// [(2 + C) * T * R], then one block per replica into out [R * (5 + C + nreg)]
template <class real>
cudaError_t launch_weather_features(const DevModel<real> &M, const double *kref_r, const int *carrier_r, int C,
                                    const int *ncar, const int32_t *reg, double *buf, double *out, cudaStream_t s);
}  // namespace esm
