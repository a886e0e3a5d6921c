// sgb_kernels.cuh -- launch interfaces of the CUDA kernels (internal).
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>

#include <vector>

#include "sgb_common.cuh"

namespace sgb {

// ------------------------------------------------------------ row filter
struct FilterArgs {
    const float *in;     // (ns, nrows)
    int ns;              // samples per row (nb)
    int nout;            // output row length (ns + extra, or the pitch); columns >= ns are zero
    long long nrows;     // nt * na * nslices
    int nt, na;          // row r -> t = r % nt, a = (r / nt) % na
    const float *wA;     // A[j*sAj + a*sAa] or null
    long long sAj, sAa;
    const float *wB;     // B[j*sBj + t*sBt] or null
    long long sBj, sBt;
    float scale;         // scalar weight (dbeta)
    unsigned *amax;      // FP32 rows only, optional: atomicMax of max |y| (bits of a non-negative float)
    // set by launch_filter_rows
    void *out;
    int kpad, nblk;      // K padded to the stage width; 256-column output blocks
    int ovec;            // 16-byte vector stores of outputs
    int *err;            // device error flags (wait timeouts)
};

// The filter as a GEMM operator: the suffix-summed Toeplitz matrix H (rows = outputs,
// K = input samples) split into np BF16 pieces in device memory, with its TMA map.
struct FilterOperator {
    int ns = 0, np = 0, kpad = 0, nblk = 0;
    DevBuf buf, err;
    CUtensorMap map;
    // tensor map of the split rows, reused while the scratch pointer and row count repeat
    mutable CUtensorMap dmap{};
    mutable const void *dmap_ptr = nullptr;
    mutable long long dmap_rows = -1;
    ~FilterOperator();
    // g: real(ifft(Hk)) (length npad); outputs up to nout_max columns per row
    int build(const std::vector<double> &g, int ns, int nout_max, int np, cudaStream_t st);
    // reads back (and reports) the kernel's error flags; synchronises st
    int check(cudaStream_t st);
};
// Output forms of launch_filter_rows: FP32 rows, BF16 rows, or FP32 pairs (y[i], y[i+1] - y[i])
// -- the FDK back-projector's layout, one 8-byte shared load per s-interpolation.  A pair's
// difference at a row's last column is 0.
enum { FILTER_OUT_F32 = 0, FILTER_OUT_BF16 = 1, FILTER_OUT_PAIR = 2 };
// Weighted, differenced, split rows go through `scratch` (grown to filter_scratch_bytes;
// pre-size it before stream capture).
size_t filter_scratch_bytes(const FilterOperator &F, long long nrows);
int launch_filter_rows(const FilterArgs &A, const FilterOperator &F, DevBuf &scratch, void *out, int out_kind,
                       cudaStream_t st);

// F16 storage form of FDK: FP32 filtered rows y (nrows = nt * na rows of `pitch` samples, ns of
// data) -> FP16 quads (8 bytes per sample, same layout), scaled by a power of two from max|y|;
// *unscale receives the inverse scale (device word).  `amax` is a device word of scratch; with
// amax_ready it already holds max |y| (the filter's epilogue folded it in) and no max pass runs.
int launch_quad_pack(const float *y, int pitch, int ns, int nt, long long nrows, void *quads, unsigned *amax,
                     float *unscale, cudaStream_t st, bool amax_ready = false);

// cuTensorMapEncodeTiled from the driver entry-point table (null when unavailable)
PFN_cuTensorMapEncodeTiled_v12000 encode_fn();

// ---------------------------------------------------- view geometry table
// per used view v (view index a = v * ia_skip): (sin, cos) in FP32 from FP64 angles.
int launch_view_trig(const double *betas_dev, int na, int ia_skip, float2 *trig, cudaStream_t st);
// streaming multiprocessors of the current device (cached per device)
int num_sms();

// -------------------------------------------------- FDK back-projection
struct FdkArgs {
    const void *proj;      // (ns, nt, na) float or bf16 filtered projections
    float *image;          // (nx, ny, nz)
    const uint8_t *mask;   // (nx, ny, nz) or null
    const float2 *trig;    // nv used views
    const float *xds, *yds, *zds;  // pixel centres / ds
    const float *zsrc;     // nv used views: source z / ds, or null
    int ns, nt, na, nx, ny, nz, nv, ia_skip;
    int pitch;             // row stride of proj in elements (>= ns)
    float ws, wt;          // (ns+1)/2 + offset_s, (nt+1)/2 + offset_t (1-based)
    float dsd_ds, dso_ds, inv_dtds;
    int is_arc;
    int is_par;            // CtPar: parallel beam (s' = x_beta, t' = z, unit weight)
    int bf16;
};
int launch_fdk_back(const FdkArgs &A, cudaStream_t st);

// ---------------------------------------------- 2D pixel-driven back-projection
struct Back2Args {
    const float *sino;     // (nb, na, nslices)
    float *image;          // (nx, ny, nslices)
    const uint8_t *mask;   // (nx, ny) or null
    const float2 *trig;    // nv used views: (sin, cos)
    const float *xds, *yds;
    int nb, na, nx, ny, nv, ia_skip, nslices;
    float wb;
    int mode;              // SGB_PAR, SGB_ARC, SGB_FLAT
    float dsd_ds, dso_ds, so_ds;
};
int launch_back2(const Back2Args &A, cudaStream_t st);

// ------------------------------------------------------- distance-driven pair
struct BddArgs {
    int nPix, nDet, na;
    const double *angle;   // device, na
    double DSD, DS0, pSize, dSize;
    int arc;               // 1: detector boundaries on the arc of radius DSD about the source
};
// scratch sizes are returned by the *_scratch functions (bytes).
size_t bdd_project_scratch(const BddArgs &G);
// project_bdd split for plans: the per-view set-up (geometry only) once, the projection per call
int launch_bdd_project_setup(const BddArgs &G, void *scratch, cudaStream_t st);
int launch_bdd_project_main(const BddArgs &G, const float *phantom, float *sino, const void *scratch,
                            cudaStream_t st);
int launch_bdd_project(const BddArgs &G, const float *phantom, float *sino, void *scratch,
                       cudaStream_t st);
size_t bdd_back_scratch(const BddArgs &G);
// backproject_bdd split the same way: the geometry table once, the sinogram's table and the
// back-projection per call
int launch_bdd_back_setup(const BddArgs &G, void *scratch, cudaStream_t st);
int launch_bdd_back_main(const BddArgs &G, const float *sino, float *image, void *scratch, cudaStream_t st);
int launch_bdd_back(const BddArgs &G, const float *sino, float *image, void *scratch,
                    cudaStream_t st);

// -------------------------------------------------------- analytic phantoms
int launch_ellipse_image(int nx, int ny, double dx, double dy, double ox, double oy, const double *ell_dev,
                         int nell, int sub, float *img, cudaStream_t st);
int launch_ellipse_sino(int kind, int nb, int na, const double *s_dev, const double *beta_dev,
                        double dso, double dsd, const double *ell_dev, int nell, float *sino,
                        cudaStream_t st);
int launch_ellipsoid_proj(int is_arc, int ns, int nt, int na, const double *s_dev,
                          const double *t_dev, const double *beta_dev, double dso, double dsd,
                          const double *ell_dev, int nell, float *proj, cudaStream_t st);

}  // namespace sgb
