// Explicit instantiation of the kernels for double.
#include "esm_kernels_impl.cuh"
#include "esm_launch.cuh"
#include "esm_linemove_impl.cuh"
#include "esm_plateau.cuh"

namespace esm {
template cudaError_t launch_scores_fused<double>(const DevModel<double> &, const double *, const double *,
                                                 const double *, const double *, double *, double *, cudaStream_t);
cudaError_t preload_score_kernels() {
    cudaFuncAttributes a;
    cudaError_t e;
    if ((e = preload_scores_f32()) != cudaSuccess) return e;
    if ((e = cudaFuncGetAttributes(&a, k_scores_fused<double>)) != cudaSuccess) return e;
    if ((e = cudaFuncGetAttributes(&a, k_score_reduce)) != cudaSuccess) return e;
    if ((e = cudaFuncGetAttributes(&a, k_score_finish<double>)) != cudaSuccess) return e;
    return cudaFuncGetAttributes(&a, k_set_kc<double>);
}
template int plateau_threads<double>(const DevModel<double> &);
template size_t plateau_scratch_reals<double>(const DevModel<double> &);
template cudaError_t launch_plateau<double>(const DevModel<double> &, const PlatMoves &, uint32_t, double *, int,
                                        unsigned long long *, cudaStream_t);
template cudaError_t launch_storage_long<double>(const DevModel<double> &, const int *, int, uint32_t, double *, int,
                                             unsigned long long *, cudaStream_t);
template size_t linemove_scratch_reals<double>(const DevModel<double> &);
template size_t linemove_smem_per_warp<double>(const DevModel<double> &);
template cudaError_t launch_class_pass<double>(const DevModel<double> &, const int *, int, const uint32_t *, int, int, double *, int, int,
                                              unsigned long long *, char *, unsigned int *, const SepLaunch &,
                                              const WaveLaunch &,
                                              cudaStream_t);
template size_t sep_region_bytes<double>(const DevModel<double> &);
template int sep_warps_per_sm<double>(const DevModel<double> &, int *);
template int linemove_blocks_per_sm<double>(const DevModel<double> &, int);
template cudaError_t launch_batch_passes<double>(const BatchModel<double> *, const BatchLaunch &, const uint32_t *,
                                                cudaStream_t);
template int batch_warps_per_sm<double>(int);
template cudaError_t launch_rebuild<double>(const DevModel<double> &, cudaStream_t);
template cudaError_t launch_score_finish<double>(const DevModel<double> &, const double *, const double *,
                                                const double *, const double *, double, double, int, double *,
                                                double *, double *, double *, cudaStream_t);
template cudaError_t launch_follow_disp<double>(const DevModel<double> &, const int *, const double *, const double *,
                                               const double *, const double *, cudaStream_t);
template cudaError_t launch_kop<double>(const DevModel<double> &, const double *, const double *, const double *,
                                       const double *, double, cudaStream_t);
template cudaError_t launch_set_kc<double>(int, const double *, const double *, const double *, const int *,
                                          const int *, double *, double *, double *, cudaStream_t);
template cudaError_t launch_weather_z<double>(const DevModel<double> &, const double *, const double *,
                                             const double *, const double *, const double *, const int *,
                                             const double *, const int *, const int *, const double *, uint64_t,
                                             uint32_t, int, cudaStream_t);
template cudaError_t launch_weather_features<double>(const DevModel<double> &, const double *, const int *, int,
                                                    const int *, const int32_t *, double *, double *, cudaStream_t);
template cudaError_t launch_compensate<double>(const DevModel<double> &, const int *, const double *, cudaStream_t);
}  // namespace esm
