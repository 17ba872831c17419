// Host entry points of the line-move kernels (esm_linemove_impl.cuh).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "esm_common.cuh"

namespace esm {
template <class real>
size_t linemove_scratch_reals(const DevModel<real> &M);  // per warp
template <class real>
size_t linemove_smem_per_warp(const DevModel<real> &M);  // bytes of one move descriptor
// the cooperative walk of the separable moves: moves whose units are storage units at distinct nodes
// and nothing else, with at least min_units units (0: none, k_move walks every move), run in
// k_move_sep on max_warps warps, their walk buffers in shared memory (in_smem) or in per-warp slabs
// of `slab` (sep_region_bytes each)
struct SepLaunch {
    int min_units, max_warps, in_smem;
    char *slab;
};
// the whole class pass in one k_move_wave launch (on = 1; not with the cooperative walk): done
// holds the moves completed per work item (max_items), err is set when a bounded wait runs out
struct WaveLaunch {
    int on;
    unsigned int *done;
    int *err;
    size_t max_items;
};
template <class real>
size_t sep_region_bytes(const DevModel<real> &M);
template <class real>
int sep_warps_per_sm(const DevModel<real> &M, int *in_smem);
// one colour class: the descriptors of its moves into descs ((natoms + nextra) descriptors), then
// per move one k_move launch (and one k_move_sep launch; the kernel that does not take the move
// returns at once); the sweep index is read on the device from *sweep (graph-capturable)
template <class real>
cudaError_t launch_class_pass(const DevModel<real> &M, const int *steps, int nsteps, const uint32_t *sweep, int cls,
                              int limit, real *scratch, int wpb, int max_warps, unsigned long long *stats,
                              char *descs, unsigned int *counters, const SepLaunch &sep, const WaveLaunch &wave,
                              cudaStream_t s);
// resident k_move warps per SM with blocks of wpb (1, 2 or 4) warps
template <class real>
int linemove_blocks_per_sm(const DevModel<real> &M, int wpb);

// ---- a batch of models whose class passes run together: per pass one descriptor launch for all
// models and one k_move_batch launch per move index, each over the tasks of every model that has
// that move (the models sorted by decreasing move count, so those are a prefix of the models)
template <class real>
struct BatchModel {
    DevModel<real> M;           // the model (move log off)
    const int *steps[3];        // the step lists of its colour classes
    int nsteps[3];
    int nmoves;                 // moves of one of its class passes (natoms + nextra)
    char *descs;                // its descriptor buffer: nmoves descriptors of stride bytes
    size_t stride;
    unsigned long long *stats;  // its move counts, laid out as a context's
};
struct BatchLaunch {
    int nm;                  // models
    int maxpass;             // colour classes per sweep, the most of any model (2, or 3 with an odd T)
    int maxmoves;            // moves per class pass of the first model (the most)
    int npass, nmove;        // the passes and the moves per pass launched (maxpass, maxmoves: all)
    const int *nact;         // host [maxmoves]: the models that have move mi (a prefix)
    int wpb, warps;          // k_move_batch: warps per block (1 or 2) and warps launched
    size_t prep_smem;        // the largest descriptor stride
    void *scratch;           // global walk slabs for the models whose buffers exceed the local arrays
    size_t scratch_per_warp; // reals of one warp's slab (0: no model needs one)
    int *pass_cls;           // device [maxpass * nm]: the class model b runs in pass p (-1: none)
    unsigned int *off;       // device [maxpass * (nm + 1)]: the item prefix over the models of pass p
    unsigned int *counters;  // device [maxpass * maxmoves]: the item counters of the launches
};
// the passes of one sweep of every model of the batch (the sweep index read from *sweep on the
// device, graph-capturable); the caching rebuild at the sweep start is the caller's
template <class real>
cudaError_t launch_batch_passes(const BatchModel<real> *bm, const BatchLaunch &bl, const uint32_t *sweep,
                                cudaStream_t s);
// resident k_move_batch warps per SM with blocks of wpb (1 or 2) warps; sets the kernels' limits
template <class real>
int batch_warps_per_sm(int wpb);

// ---- storage multiscale sweep (esm_plateau.cuh)
#define ESM_PLAT_MAXU 32  // units of one plateau move (a cell-class aggregate)
#define ESM_PLAT_MAXK 8   // dispatchable units at one node taking part in the compensation
// the moves of one class pass, drawn on the host
struct PlatMoves {
    int L, o, cls, li, nb;      // length, offset, block parity, length index, blocks of the class
    int nu[8];                  // units per move
    int j[8][ESM_PLAT_MAXU];    // storage unit indices (into stor)
};
template <class real>
int plateau_threads(const DevModel<real> &M);  // resident threads of k_plateau
template <class real>
size_t plateau_scratch_reals(const DevModel<real> &M);  // global scratch per thread (0: local arrays)
template <class real>
cudaError_t launch_plateau(const DevModel<real> &M, const PlatMoves &mv, uint32_t sweep, real *scratch, int threads,
                           unsigned long long *stats, cudaStream_t s);
// ---- long-range storage sweep: per unit [stor index, moves, (L, a) per move], at most 5 moves
#define ESM_SL_STRIDE 12
template <class real>
cudaError_t launch_storage_long(const DevModel<real> &M, const int *plan, int nunits, uint32_t sweep, real *scratch,
                                int threads, unsigned long long *stats, cudaStream_t s);
}  // namespace esm
