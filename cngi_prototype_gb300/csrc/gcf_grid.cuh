// Mosaic gridding kernel shared by the translation units that instantiate it
// (gcf_grid_lo.cu, gcf_grid_mid.cu, gcf_grid_hi.cu) and the host set-up
// in gcf.cu.
#pragma once
#include "ngg_internal.cuh"

namespace ngg {

constexpr int MAXS = 31;    // largest support (one lane per column class)
constexpr int SP = 32;      // columns per tap row of the reorganised table (one per lane)
constexpr int GCH = 128;    // time steps per warp item (decoded 32 at a time)

struct GChan {
    double su, sv;
    float suh, sul, svh, svl;
};

struct GArgs {
    const float2 *vis;
    const float *weight;
    const double *uvw;
    const float4 *uvs;
    const GChan *chan;
    const int32_t *field_index, *cfb_map, *cfc_map, *cfp_map;
    const float *ckt;
    const float2 *gx, *gy, *hx, *hy;
    const double2 *ex64, *ey64;
    const double2 *nrm;
    float2 *grid;
    double *sum_weight;
    int64_t T, B, C, P, nu, nv, ncfb, ncfc, ncfp, ncf, R0, R1;
    int os0, os1, S, maxsup, nk, n_img, continuum, fftl, nf;
};

// launch k_grid_gcf<DATA, S> for odd S: 1-15 (gcf_grid_lo.cu), 17-23
// (gcf_grid_mid.cu), 25-31 (gcf_grid_hi.cu)
int launch_grid_gcf_lo(const GArgs &a, bool data, unsigned blocks, cudaStream_t s);
int launch_grid_gcf_mid(const GArgs &a, bool data, unsigned blocks, cudaStream_t s);
int launch_grid_gcf_hi(const GArgs &a, bool data, unsigned blocks, cudaStream_t s);

}  // namespace ngg
