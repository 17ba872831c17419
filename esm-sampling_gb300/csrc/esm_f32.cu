// Explicit instantiation of the kernels for float.
#include "esm_kernels_impl.cuh"
#include "esm_launch.cuh"
#include "esm_linemove_impl.cuh"
#include "esm_plateau.cuh"

namespace esm {
cudaError_t launch_scores_f32(const DevModel<float> &Mf, const DevModel<double> &Md, double *partial, double *sums,
                              cudaStream_t s) {
    return launch_scores_f32_t<0>(Mf, Md, partial, sums, s);
}
cudaError_t preload_scores_f32() { return preload_scores_f32_t<0>(); }
template int plateau_threads<float>(const DevModel<float> &);
template size_t plateau_scratch_reals<float>(const DevModel<float> &);
template cudaError_t launch_plateau<float>(const DevModel<float> &, const PlatMoves &, uint32_t, float *, int,
                                        unsigned long long *, cudaStream_t);
template cudaError_t launch_storage_long<float>(const DevModel<float> &, const int *, int, uint32_t, float *, int,
                                             unsigned long long *, cudaStream_t);
template size_t linemove_scratch_reals<float>(const DevModel<float> &);
template size_t linemove_smem_per_warp<float>(const DevModel<float> &);
template cudaError_t launch_class_pass<float>(const DevModel<float> &, const int *, int, const uint32_t *, int, int, float *, int, int,
                                              unsigned long long *, char *, unsigned int *, const SepLaunch &,
                                              const WaveLaunch &,
                                              cudaStream_t);
template size_t sep_region_bytes<float>(const DevModel<float> &);
template int sep_warps_per_sm<float>(const DevModel<float> &, int *);
template int linemove_blocks_per_sm<float>(const DevModel<float> &, int);
template cudaError_t launch_batch_passes<float>(const BatchModel<float> *, const BatchLaunch &, const uint32_t *,
                                                cudaStream_t);
template int batch_warps_per_sm<float>(int);
template cudaError_t launch_rebuild<float>(const DevModel<float> &, cudaStream_t);
template cudaError_t launch_score_finish<float>(const DevModel<float> &, const double *, const double *,
                                                const double *, const double *, double, double, int, double *,
                                                double *, double *, double *, cudaStream_t);
template cudaError_t launch_follow_disp<float>(const DevModel<float> &, const int *, const double *, const double *,
                                               const double *, const double *, cudaStream_t);
template cudaError_t launch_kop<float>(const DevModel<float> &, const double *, const double *, const double *,
                                       const double *, double, cudaStream_t);
template cudaError_t launch_set_kc<float>(int, const double *, const double *, const double *, const int *,
                                          const int *, float *, float *, float *, cudaStream_t);
template cudaError_t launch_weather_z<float>(const DevModel<float> &, const double *, const double *,
                                             const double *, const double *, const double *, const int *,
                                             const double *, const int *, const int *, const double *, uint64_t,
                                             uint32_t, int, cudaStream_t);
template cudaError_t launch_weather_features<float>(const DevModel<float> &, const double *, const int *, int,
                                                    const int *, const int32_t *, double *, double *, cudaStream_t);
template cudaError_t launch_compensate<float>(const DevModel<float> &, const int *, const float *, cudaStream_t);
}  // namespace esm
