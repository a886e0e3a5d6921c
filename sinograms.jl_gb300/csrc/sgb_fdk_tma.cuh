// sgb_fdk_tma.cuh -- launch interface of the TMA-staged FDK back-projector (internal).
#pragma once
#include <cuda.h>

#include "sgb_common.cuh"

namespace sgb {

struct FdkTmaArgs {
    const float2 *trig;     // nv used views: (sin, cos)
    const float *zsrc;      // nv used views: source z / ds (helical shift), or null (z_src = 0)
    float *image;           // (nx, ny, nz)
    const uint8_t *mask;    // (nx, ny, nz) or null
    int *err;               // device error flags: 1 box too small, 2 wait timeout, 4 drain timeout
    int ns, nt, na, nx, ny, nz, nv, ia_skip;
    float ws, wt, dsd_ds, dso_ds, inv_dtds;
    float x0, dx, y0, dy, z0, dz;  // uniform voxel-centre axes / ds
    int is_arc;
    int zu;                 // voxels per thread along z (16 or 32)
    int elem_bytes;         // 8 (FP32 pairs or FP16 quads), 4 (FP32) or 2 (BF16) per filtered sample
    int quad;               // 1: 8-byte samples are FP16 quads scaled by one power of two (F16 form)
    const float *qscale;    // F16 form: device word with the factor that undoes the quads' scale
    int align;              // TMA x-coordinate alignment in elements
    int W, H, box_bytes;    // staged box (samples) and its shared-memory footprint
    int vps;                // views per pipeline stage (4, or 2 for large boxes)
    int v0;                 // first view of this launch (views v0 .. v0 + nv - 1)
    int accum;              // 1: add to the volume (a later pass over views), 0: overwrite
    int passes;             // launches the views are split over (chosen by the plan's autotuner)
    int nstage;             // batched scans: stages of the box ring (4, or 2 for tall boxes)
};

// Batched persistent back-projection: per-scan arguments in device memory, tensor maps in
// the kernel parameter block (at most kMaxBatch scans per launch).
constexpr int kMaxBatch = 64;
// persistent launches of one batch: box classes of (sample bytes 8/4/2) x (width 32/64/128) x
// (z unroll 16/32/64) that occur, at most this many; each has its own work counter
constexpr int kMaxBatchClasses = 16;
// stages of the box ring of the TMA-staged back-projectors (batched scans with tall boxes may
// take a 2-stage ring instead)
constexpr int kNStageDefault = 4;
struct FdkBatchMaps {
    CUtensorMap m[kMaxBatch];
};
struct FdkBatchArgs {
    const FdkTmaArgs *scans;  // device array [nscans]
    const int2 *work;         // device array [nwork]: (scan, tile) in execution order
    int *counter;             // device work counter (zero before the launch)
    int *err;                 // device error flags
    int nscans, nwork;
    int W;                    // common compile-time box width (32 or 64)
    int box_bytes;            // largest box of the batch
    int elem_bytes;
    int quad;                 // 8-byte samples are FP16 quads (F16 form)
    int vps;                  // views per pipeline stage (4, 2 or 1)
    int zu;                   // voxels per thread along z of every scan in the launch (16, 32, 64)
    int nstage;               // stages of the box ring (4; 2 with one view per stage)
};
size_t fdk_batch_smem(const FdkBatchArgs &B);
int fdk_batch_ctas_per_sm(const FdkBatchArgs &B);
int launch_fdk_batch(const FdkBatchArgs &B, const FdkBatchMaps &maps, int nctas, cudaStream_t st);
// one storage form each (sgb_fdk_batch_<form>.cu)
int launch_fdk_batch_pair(const FdkBatchArgs &B, const FdkBatchMaps &maps, int nctas, cudaStream_t st);
int launch_fdk_batch_f32(const FdkBatchArgs &B, const FdkBatchMaps &maps, int nctas, cudaStream_t st);
int launch_fdk_batch_bf16(const FdkBatchArgs &B, const FdkBatchMaps &maps, int nctas, cudaStream_t st);
int launch_fdk_batch_quad(const FdkBatchArgs &B, const FdkBatchMaps &maps, int nctas, cudaStream_t st);
int fdk_batch_ctas_per_sm_quad(const FdkBatchArgs &B);
int fdk_batch_ctas_per_sm_pair(const FdkBatchArgs &B);
int fdk_batch_ctas_per_sm_f32(const FdkBatchArgs &B);
int fdk_batch_ctas_per_sm_bf16(const FdkBatchArgs &B);

// Sizes the detector box over every (tile, view) of the geometry (device pre-pass).
int fdk_tma_prepare(FdkTmaArgs &A, int *ext_dev, cudaStream_t st);
// Picks views-per-stage for the staged box; false when no ring fits shared memory.
bool fdk_tma_choose(FdkTmaArgs &A);
// The chosen ring leaves room for two CTAs per SM.
bool fdk_tma_fits_two_ctas(const FdkTmaArgs &A);
// one view per stage in a ring of `nstage` stages lets two CTAs share an SM
bool fdk_tma_fits_two_ctas_ring(const FdkTmaArgs &A, int nstage);
size_t fdk_tma_smem(const FdkTmaArgs &A, int vps, int nstage);
// 3D tensor map over the filtered projections (pitch, nt, na).
int fdk_tma_encode(const FdkTmaArgs &A, const void *filt, int pitch, CUtensorMap *map);
int launch_fdk_tma(const FdkTmaArgs &A, const CUtensorMap &map, cudaStream_t st);
// one storage form each (sgb_fdk_tma_<form>.cu)
int launch_fdk_tma_pair_flat(const FdkTmaArgs &A, const CUtensorMap &map, cudaStream_t st);
int launch_fdk_tma_pair_arc(const FdkTmaArgs &A, const CUtensorMap &map, cudaStream_t st);
int launch_fdk_tma_quad_flat(const FdkTmaArgs &A, const CUtensorMap &map, cudaStream_t st);
int launch_fdk_tma_quad_arc(const FdkTmaArgs &A, const CUtensorMap &map, cudaStream_t st);
int launch_fdk_tma_f32(const FdkTmaArgs &A, const CUtensorMap &map, cudaStream_t st);
int launch_fdk_tma_bf16(const FdkTmaArgs &A, const CUtensorMap &map, cudaStream_t st);

}  // namespace sgb
