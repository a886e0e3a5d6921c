// sgb_fdk_tma.cuh -- launch interface of the TMA-staged FDK back-projector (internal).
#pragma once
#include <cuda.h>

#include "sgb_common.cuh"

namespace sgb {

struct FdkTmaArgs {
    const float2 *trig;     // nv used views: (sin, cos)
    float *image;           // (nx, ny, nz)
    const uint8_t *mask;    // (nx, ny, nz) or null
    int *err;               // device error flags: 1 box too small, 2 wait timeout, 4 drain timeout
    int ns, nt, na, nx, ny, nz, nv, ia_skip;
    float ws, wt, dsd_ds, dso_ds, inv_dtds;
    float x0, dx, y0, dy, z0, dz;  // uniform voxel-centre axes / ds
    int is_arc;
    int zu;                 // voxels per thread along z (16 or 32)
    int elem_bytes;         // 4 (fp32) or 2 (bf16) filtered projections
    int align;              // TMA x-coordinate alignment in elements
    int W, H, box_bytes;    // staged box (samples) and its shared-memory footprint
};

// Sizes the detector box over every (tile, view) of the geometry (device pre-pass).
int fdk_tma_prepare(FdkTmaArgs &A, int *ext_dev, cudaStream_t st);
bool fdk_tma_usable(const FdkTmaArgs &A);
size_t fdk_tma_smem(const FdkTmaArgs &A, int vps, int nstage);
// 3D tensor map over the filtered projections (pitch, nt, na).
int fdk_tma_encode(const FdkTmaArgs &A, const void *filt, int pitch, CUtensorMap *map);
int launch_fdk_tma(const FdkTmaArgs &A, const CUtensorMap &map, cudaStream_t st);

}  // namespace sgb
