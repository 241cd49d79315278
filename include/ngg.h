/*
 * ngg.h -- C ABI of the GB300-native ngcasa imaging hot path (libngg.so).
 *
 * Every entry point takes device pointers that the caller owns, a CUDA stream
 * (cudaStream_t passed as void*, NULL = legacy default stream) and returns an
 * NGG_* status. Work is enqueued on the stream; results are valid once the
 * stream has reached that point. Array layouts follow the reference's numpy
 * arrays (C order): visibilities (time, baseline, chan, pol), uvw
 * (time, baseline, 3), grids (chan, pol, u, v), images (l, m, chan, pol) --
 * the same layouts its per-chunk numpy functions take and return.
 *
 * Thread safety: calls on different streams may run concurrently; the cuFFT
 * plan cache is internally locked.
 */
#ifndef NGG_H
#define NGG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define NGG_OK 0
#define NGG_ERR_INVALID 1     /* bad argument (shape, null pointer, range)      */
#define NGG_ERR_NOMEM 2       /* device allocation of scratch failed           */
#define NGG_ERR_CUDA 3        /* a CUDA runtime / cuFFT call failed            */
#define NGG_ERR_UNSUPPORTED 4 /* valid request this build does not implement   */
#define NGG_ERR_TIMEOUT 5     /* a bounded device-side wait ran out            */

/* ---- enumerations ------------------------------------------------------ */
#define NGG_MODE_DATA 0   /* grid vis*weight into a complex grid               */
#define NGG_MODE_PSF 1    /* grid weight into a real grid                      */

#define NGG_CHAN_CUBE 0       /* one image channel per visibility channel      */
#define NGG_CHAN_CONTINUUM 1  /* all channels into image channel 0             */

#define NGG_LAYOUT_NATURAL 0  /* grid[c,p,u,v] as the reference returns it     */
#define NGG_LAYOUT_FFT 1      /* each plane ifftshift-ed: cell (u,v) stored at
                                 ((u - Nu/2) mod Nu, (v - Nv/2) mod Nv), the
                                 input order of an unshifted inverse FFT        */

#define NGG_WEIGHTING_NATURAL 0
#define NGG_WEIGHTING_UNIFORM 1
#define NGG_WEIGHTING_BRIGGS 2
#define NGG_WEIGHTING_BRIGGS_ABS 3

/* Library version, e.g. 100 for 0.1.0. */
int ngg_version(void);
/* Message of the last failing call on this host thread ("" when none). */
const char *ngg_last_error(void);

/* ---- standard (prolate-spheroidal) gridder -------------------------------
 * Replaces _standard_grid_numpy_wrap / _standard_grid_psf_numpy_wrap and
 * the loop nest _standard_grid_jit
 * (ngcasa/imaging/_imaging_utils/_standard_grid.py:123-236, :242-371).
 *
 * delta_lm is grid_parms['cell_size'] after _check_grid_parms, i.e. in
 * radians with delta_lm[0] already negated (_check_imaging_parms.py:38-39).
 * cgk_1D is the oversampled half-kernel table of length
 * oversampling*(support/2+1) (_create_prolate_spheroidal_kernel_1D).
 * weight holds the imaging weights (float32, same shape as vis).
 * Output grid: complex64 (DATA) or float32 (PSF), shape
 * (n_chan_img, n_pol, n_u, n_v) where n_chan_img = n_chan (cube) or 1
 * (continuum); sum_weight float64 (n_chan_img, n_pol). Both are overwritten.
 * With NGG_LAYOUT_FFT the grid is always complex64 (a PSF grid then has zero
 * imaginary parts), ready for ngg_fft_correct.
 * Taps and accumulation are FP32; cell and oversampling indices are the ones
 * the reference's FP64 arithmetic produces (bit-exact). support must be 7
 * and oversampling in [1, 1000] in this build.
 */
typedef struct NggGridArgs {
    int mode;          /* NGG_MODE_DATA | NGG_MODE_PSF                         */
    int chan_mode;     /* NGG_CHAN_CUBE | NGG_CHAN_CONTINUUM                   */
    int layout;        /* NGG_LAYOUT_NATURAL | NGG_LAYOUT_FFT                  */
    int support;
    int oversampling;
    int reserved0;
    int64_t n_time, n_baseline, n_chan, n_pol;
    int64_t n_u, n_v;  /* padded grid size (image_size_padded)                */
    double delta_lm[2];
    const void *vis;      /* complex64 (T,B,C,P); NULL for PSF                 */
    const double *uvw;    /* float64 (T,B,3) metres                            */
    const float *weight;  /* float32 (T,B,C,P)                                 */
    const double *freq;   /* float64 (C) Hz                                    */
    const double *cgk_1D; /* float64 (oversampling*(support/2+1))              */
    void *grid;           /* complex64 / float32 (Cimg,P,Nu,Nv)                */
    double *sum_weight;   /* float64 (Cimg,P)                                  */
} NggGridArgs;

int ngg_grid_ps(const NggGridArgs *args, void *stream);

/* ngg_grid_ps_chunk: the same gridding of channels [chan_offset,
 * chan_offset + n_chan) of larger input arrays: args->vis and args->weight
 * are (T,B,n_chan_total,P) (the reference's whole-cube arrays), args->freq
 * and the outputs describe only the n_chan channels of this call (the
 * per-chunk call of _graph_standard_grid, _standard_grid.py:62-75, without
 * slicing the inputs). vis and weight may be device memory or pinned host
 * memory; pinned host memory is read in place by the packing kernel over the
 * host link (no staging copy). Pageable host memory is refused
 * (NGG_ERR_INVALID), as it is by ngg_grid_ps. */
int ngg_grid_ps_chunk(const NggGridArgs *args, int64_t chan_offset, int64_t n_chan_total, void *stream);

/* ngg_grid_ps_weighted: ngg_grid_ps with the imaging weights formed inside
 * the packing pass instead of read from an IMAGING_WEIGHT array, and with
 * flags applied to the visibilities -- the per-channel-chunk pipeline of
 * synthesis_imaging_cube (ngcasa/imaging/synthesis_imaging_cube.py:170-308:
 * vis[flag] = NaN, _make_imaging_weight_chunk, then the PSF and image
 * gridding) in one pass per grid. args->weight holds the natural weights
 * (DATA_WEIGHT). With density non-NULL each weight becomes, as in
 * _standard_imaging_weight_degrid_jit (_standard_grid.py:466-518), the
 * two-pol average divided by f0*W + f1 at the step's nearest cell of the
 * unpadded density grid (0 outside it); density and factors are the outputs
 * of ngg_grid_density and ngg_briggs_factors for the same channels. With
 * density NULL the weights are used as given (natural weighting). flag, if
 * non-NULL, marks visibilities left out of DATA-mode grids (the reference
 * sets them to NaN; its PSF and weight density still use their weights).
 * Same outputs, ownership and errors as ngg_grid_ps. */
typedef struct NggImagingWeights {
    const float *density;        /* float32 (Cimg, n_u, n_v) or NULL        */
    const double *factors;       /* float64 (2, Cimg) Briggs f0, f1         */
    int64_t n_u, n_v;            /* density grid = the unpadded image size  */
    const uint8_t *flag;         /* uint8 (T,B,C,P), nonzero = flagged      */
} NggImagingWeights;
int ngg_grid_ps_weighted(const NggGridArgs *args, const NggImagingWeights *iw, void *stream);

/* Cell and oversampling-offset indices as the gridder's packing pass
 * computes them (one certified FP32-pair floor of 2 (u_pos + 0.5) os, then
 * the two-floor FP32-pair chain, then FP64 near rounding boundaries; every
 * path gives the FP64 chain's integers): for each uvw row r and
 * channel c, idx[(r*n_chan + c)*4 + {0,1,2,3}] = (cu, cv, ou, ov), with
 * cu = int(u_pos + 0.5), ou = floor((cu - u_pos)*oversampling + 0.5) and
 * likewise for v (_standard_grid.py:299-324), mirrored (-u, -v) when
 * mirror != 0. n_fallback (device int64, may be NULL) receives the number of
 * coordinates that needed the FP64 path. For verification and tooling. */
int ngg_cell_indices(int64_t n_rows, int64_t n_chan, const double *uvw, const double *freq,
                     int64_t n_u, int64_t n_v, const double delta_lm[2], int oversampling,
                     int mirror, int32_t *idx, long long *n_fallback, void *stream);

/* ---- imaging weights ------------------------------------------------------
 * Weight-density grid: replaces the do_imaging_weight branch of
 * _standard_grid_jit as called by calc_briggs_weights
 * (make_imaging_weight.py:153-161; _standard_grid.py:327-333, 349-369):
 * unpadded n_u x n_v grid, nearest cell, the mirrored cell (-u,-v) also
 * incremented, weights of two or more pols averaged over pols 0 and 1.
 * Because every pol then receives the same value, the reference's
 * (chan, pol, u, v) density grid has identical planes for all pols; this call
 * writes that plane once: density float32 (n_chan_img, n_u, n_v) and
 * density_sum_weight float64 (n_chan_img) (which the reference also stores
 * per pol, identically). Mirrored cells that fall off the grid (only
 * possible for centre cells 0 or 1 at the edge) are dropped.
 */
int ngg_grid_density(int chan_mode, int64_t n_time, int64_t n_baseline, int64_t n_chan,
                     int64_t n_pol, int64_t n_u, int64_t n_v, const double delta_lm[2],
                     const double *uvw, const float *weight, const double *freq,
                     float *density, double *density_sum_weight, void *stream);

/* Briggs / uniform factors: replaces calculate_briggs_parms
 * (make_imaging_weight.py:198-213). factors float64 (2, n_chan_img):
 * briggs: f0 = (5*10^-robust)^2 / (sum(W^2)/sum_weight), f1 = 1;
 * uniform: f0 = 1, f1 = 0; briggs_abs: f0 = robust^2, f1 = 2*noise^2 (the
 * documented intent; the reference's branch raises NameError). */
int ngg_briggs_factors(int weighting, double robust, double briggs_abs_noise,
                       int64_t n_chan_img, int64_t n_u, int64_t n_v, const float *density,
                       const double *density_sum_weight, double *factors, void *stream);

/* Imaging-weight lookup: replaces _standard_imaging_weight_degrid_numpy_wrap
 * and _standard_imaging_weight_degrid_jit (_standard_grid.py:443-518).
 * imaging_weight float32 (T,B,C,P): two-pol average of weight divided by
 * f0*W[cell]+f1 where the pol's own weight and W are finite and non-zero;
 * 0 where the nearest cell is off the grid or uvw is NaN. */
int ngg_weight_lookup(int chan_mode, int64_t n_time, int64_t n_baseline, int64_t n_chan,
                      int64_t n_pol, int64_t n_u, int64_t n_v, const double delta_lm[2],
                      const double *uvw, const float *weight, const double *freq,
                      const float *density, const double *factors, float *imaging_weight,
                      void *stream);

/* ---- FFT, crop and gridding correction ------------------------------------
 * Replaces the tail of make_image / make_psf (make_image.py:116-130,
 * make_psf.py:117-131): image = Re(fftshift(ifft2(ifftshift(grid))))*Nu*Nv
 * cropped to the centre (n_l, n_m) window (_remove_padding.py:20-31),
 * divided by sum_weight (0 -> 1) and by correction[l,m] (the cropped
 * grid-correction image). grid is a stack of n_chan_img*n_pol complex64
 * planes in NGG_LAYOUT_FFT order; it is transformed IN PLACE (destroyed).
 * image float64 (n_l, n_m, n_chan_img, n_pol).
 * correction float64 (n_l, n_m); sum_weight float64 (n_chan_img, n_pol). */
int ngg_fft_correct(void *grid, int64_t n_chan_img, int64_t n_pol,
                    int64_t n_u, int64_t n_v, int64_t n_l, int64_t n_m,
                    const double *sum_weight, const double *correction, double *image,
                    void *stream);

/* As ngg_fft_correct with the inverse transform in double precision
 * (complex128 working planes in library scratch; grid is left unchanged).
 * The FP32 transform's rounding, amplified by 1/correction towards the image
 * edge (the correction falls to ~1.5e-3 in the corners), puts a floor of
 * ~6e-6 of the peak under the image error; this variant removes it at
 * ~15-25x the transform time (GB300 executes FP64 at a small fraction of
 * its FP32 rate). Same reference lines as ngg_fft_correct. */
int ngg_fft_correct_f64(const void *grid, int64_t n_chan_img, int64_t n_pol,
                        int64_t n_u, int64_t n_v, int64_t n_l, int64_t n_m,
                        const double *sum_weight, const double *correction, double *image,
                        void *stream);

/* ---- degridding: the exact adjoint of the imaging operator ---------------
 * The reference has no visibility degridder (_graph_standard_degrid prints
 * "Degridding of visibilities and psf still needs to be implemented",
 * _standard_grid.py:429-430); these two calls are the adjoints of
 * ngg_fft_correct and of ngg_grid_ps (DATA mode) so that
 * make_image = fft_correct . grid_ps has the transpose
 * degrid_ps . fft_correct_adjoint (real inner product on images, complex on
 * visibilities).
 *
 * ngg_fft_correct_adjoint: image (n_l, n_m, n_chan_img, n_pol), float32 or
 * float64 (image_is_f64), is divided by sum_weight (0 -> 1) and correction,
 * placed at the cropped window of zeroed padded planes in NGG_LAYOUT_FFT
 * order, and forward-transformed (unnormalised, e^{-i}) in place: grid
 * complex64 (n_chan_img, n_pol, n_u, n_v) in NGG_LAYOUT_FFT order.
 *
 * ngg_degrid_ps: vis[t,b,c,p] = weight[t,b,c,p] * sum_taps conv * grid[cell]
 * over the same 7x7 footprint, cells and oversampling offsets as
 * ngg_grid_ps; 0 where the footprint leaves the grid or uvw is NaN. weight
 * may be NULL (all ones). grid layout given by `layout`. */
typedef struct NggDegridArgs {
    int chan_mode;
    int layout;
    int support;
    int oversampling;
    int64_t n_time, n_baseline, n_chan, n_pol;
    int64_t n_u, n_v;
    double delta_lm[2];
    const void *grid;     /* complex64 (Cimg,P,Nu,Nv)                           */
    const double *uvw;    /* float64 (T,B,3)                                    */
    const float *weight;  /* float32 (T,B,C,P) or NULL                          */
    const double *freq;   /* float64 (C)                                        */
    const double *cgk_1D; /* float64 (oversampling*(support/2+1))               */
    void *vis;            /* complex64 (T,B,C,P) output                         */
} NggDegridArgs;

int ngg_degrid_ps(const NggDegridArgs *args, void *stream);

/* ngg_predict_ps: model visibilities from a model grid (the degridding step
 * of predict_modelvis_image, ngcasa/imaging/predict_modelvis_image.py:20-39,
 * a stub in the reference that lists normalise, stokes_to_corr, Fourier
 * transform and degrid). Same arguments and footprint as ngg_degrid_ps; each
 * visibility is divided by its kernel sum (sum conv_u)(sum conv_v), so a
 * model grid from ngg_fft_correct_adjoint with sum_weight 1 gives
 * vis = sum_pixels I exp(-2 pi i (u l + v m)) up to the kernel's aliasing and
 * the oversampled table's quantisation. weight NULL predicts every row. */
int ngg_predict_ps(const NggDegridArgs *args, void *stream);

/* ngg_degrid_ps_noalloc: the same result as ngg_degrid_ps, for callers that
 * must not have the library allocate device memory (e.g. a host application
 * that owns and budgets all device memory itself). No counterpart in the
 * reference. Its scratch is a fixed array inside the library (present on
 * every GPU that loads libngg.so until the process exits), so sizes are
 * limited: n_time*n_baseline <= NGG_NOALLOC_MAX_ROWS and
 * n_chan <= NGG_NOALLOC_MAX_CHAN, else NGG_ERR_INVALID. The first call on a
 * device (and the first after its context was replaced, e.g. by
 * cudaDeviceReset) looks up that array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * Calls share the array: calls whose GPU work overlaps (e.g. on two streams)
 * corrupt each other. */
#define NGG_NOALLOC_MAX_ROWS 1048576
#define NGG_NOALLOC_MAX_CHAN 16384
int ngg_degrid_ps_noalloc(const NggDegridArgs *args, void *stream);

int ngg_fft_correct_adjoint(const void *image, int image_is_f64, int64_t n_chan_img, int64_t n_pol,
                            int64_t n_u, int64_t n_v, int64_t n_l, int64_t n_m,
                            const double *sum_weight, const double *correction, void *grid,
                            void *stream);

/* ---- mosaic (aperture-projection) gridding with a GCF table ---------------
 * Replaces _aperture_grid_numpy_wrap / _aperture_psf_grid_numpy_wrap /
 * _aperture_grid_jit (ngcasa/imaging/_imaging_utils/_aperture_grid.py:294-513)
 * and _aperture_weight_grid_jit (:146-291).
 *
 * conv_kernel: float64 (n_cf_baseline, n_cf_chan, n_cf_pol, R0, R1), the
 * CONV_KERNEL (or WEIGHT_CONV_KERNEL) table of make_gridding_convolution_function;
 * support: int32 (n_cf_baseline, n_cf_chan, n_cf_pol, 2). The phase gradient
 * of field f is exp(i*(x*phase_slope[f,0] + y*phase_slope[f,1])) with (x, y)
 * the table offsets from its centre (R0/2, R1/2) -- the table
 * make_phase_gradient builds (make_gridding_convolution_function.py:331-359).
 * field_index: int32 (T, B), the index into the field list of each row's
 * FIELD_ID, or -1 to skip the row. Maps: cf_baseline_map int32 (B),
 * cf_chan_map int32 (C), cf_pol_map int32 (P). weight = imaging weights.
 * Taps: table[cfb,cfc,cfp, os0*iu + off_u + R0/2, os1*iv + off_v + R1/2] times
 * the phase gradient, |iu|,|iv| <= support/2; a row is skipped when any cell
 * within max(support) of its centre leaves the grid (the reference's rule).
 * sum_weight: weight*Re(norm^2) (DATA) or weight*Re(norm) (PSF), norm = sum
 * of the row's complex taps. Grid complex64 (Cimg, P, Nu, Nv), overwritten.
 * ngg_grid_gcf_weight: the weight grid of make_mosaic_pb: every tap placed
 * at the grid centre, sum_weight += weight*Re(norm). */
typedef struct NggGcfArgs {
    int mode;          /* NGG_MODE_DATA | NGG_MODE_PSF (ignored by the weight grid) */
    int chan_mode;
    int layout;
    int oversampling[2];
    int n_field;
    int64_t n_time, n_baseline, n_chan, n_pol;
    int64_t n_u, n_v;
    double delta_lm[2];
    int64_t n_cf_baseline, n_cf_chan, n_cf_pol;
    int64_t conv_size[2];        /* R0, R1 */
    const void *vis;             /* complex64 (T,B,C,P); NULL for PSF / weight */
    const double *uvw;           /* float64 (T,B,3)            */
    const float *weight;         /* float32 (T,B,C,P)          */
    const double *freq;          /* float64 (C)                */
    const int32_t *field_index;  /* int32 (T,B)                */
    const int32_t *cf_baseline_map, *cf_chan_map, *cf_pol_map;
    const double *conv_kernel;   /* float64 (ncfb,ncfc,ncfp,R0,R1) */
    const int32_t *support;      /* int32 (ncfb,ncfc,ncfp,2)   */
    const double *phase_slope;   /* float64 (n_field, 2)       */
    void *grid;                  /* complex64 (Cimg,P,Nu,Nv)   */
    double *sum_weight;          /* float64 (Cimg,P)           */
} NggGcfArgs;

int ngg_grid_gcf(const NggGcfArgs *args, void *stream);
int ngg_grid_gcf_weight(const NggGcfArgs *args, void *stream);

/* GCF generation helpers (make_gridding_convolution_function.py:181-246 with
 * _make_pb_symmetric.py:79-235): for every antenna pair and PB frequency,
 * the pair's voltage pattern product on an n0 x n1 grid of `cell` (radians,
 * the image cell times the GCF oversampling) centred at (c0, c1) -- Airy
 * disk of dish and blockage diameters, CASA form (casa_model = 1) or the
 * textbook obscured form (0) -- and the real part of its centred FFT,
 * real(fftshift(fft2(ifftshift(pattern^ipower)))) for ipower 1 (conv_kernel)
 * and 2 (weight_conv_kernel), in FP64. pairs: int32 (n_pairs, 2) indices
 * into the diameter lists. Outputs float64 (n_pairs, n_freq, n0, n1). */
int ngg_gcf_kernels(int casa_model, int64_t n_types, const double *dish_diameters,
                    const double *blockage_diameters, int64_t n_pairs, const int32_t *pairs,
                    int64_t n_freq, const double *freq, int64_t n0, int64_t n1,
                    const double cell[2], int64_t c0, int64_t c1, double *conv_kernel,
                    double *weight_conv_kernel, void *stream);

/* Primary beam of each dish type on the image grid, as synthesis_imaging_cube
 * makes it (_make_pb, synthesis_imaging_cube.py:262-277, with
 * _airy_disk / _casa_airy_disk, _make_pb_symmetric.py:26-128): the Airy
 * voltage pattern (CASA form for casa_model = 1, textbook obscured form for
 * 0) of dish and blockage diameters at radius sqrt(x^2+y^2) * 2 pi f / c *
 * dish / 2, x = (i - c0) cell[0], y = (j - c1) cell[1], raised to ipower
 * (2: the power pattern), with the centre pixel exactly 1. dish, block:
 * float64 (n_types) device arrays; freq float64 (n_freq). Output float64
 * (n0, n1, n_freq, n_types). */
int ngg_primary_beam(int casa_model, int64_t n_types, const double *dish_diameters,
                     const double *blockage_diameters, int64_t n_freq, const double *freq, int64_t n0, int64_t n1,
                     const double cell[2], int64_t c0, int64_t c1, int ipower, double *out, void *stream);

/* Mosaic normalisation (make_image_with_gcf / make_psf_with_gcf through
 * _normalize, ngcasa/imaging/_imaging_utils/_normalize.py:14-90, forward
 * direction), in place on image float64 (n_l, n_m, n_planes) that already
 * holds Re(FFT^-1 grid) * Nu*Nv / sum_weight (ngg_fft_correct with a
 * correction of ones): image / (osc * (ps_corr * norm_image)) with
 * osc(l, m) = sinc((l - n_l/2) / (n_l os0)) * sinc((m - n_m/2) / (n_m os1)),
 * ps_corr (n_l, n_m) or NULL (ones), norm_image (n_l, n_m, n_planes) or NULL
 * (ones: norm_type 'none'; PB for 'flat_noise', WEIGHT_PB for 'flat_sky');
 * then 0 where pb < pb_limit (pb_limit > 0 and pb not NULL), then rounded
 * through float32 if single_precision. If centre is not NULL every plane is
 * finally divided by its value at (centre[0], centre[1]) (the PSF,
 * make_psf_with_gcf.py:99). */
int ngg_mosaic_normalize(double *image, int64_t n_l, int64_t n_m, int64_t n_planes,
                         const double *ps_corr, const double *norm_image, const double *pb,
                         double pb_limit, const int oversampling[2], int single_precision,
                         const int64_t *centre, void *stream);

/* out[i] = sqrt(|x[i]|): the mosaic PB from WEIGHT_PB (make_mosaic_pb.py:150). */
int ngg_sqrt_abs(const double *x, int64_t n, double *out, void *stream);

/* ---- learned GCF: coordinate MLP ------------------------------------------
 * No counterpart in the reference (it has no learned component). A small
 * network stands in for the CONV_KERNEL table of
 * make_gridding_convolution_function (make_gridding_convolution_function.py:
 * 164-311): inputs z = (x, y, f) scaled to about [-1, 1] (table offsets
 * from the centre and frequency), c = (x, y, r = |(x, y)|, f), Fourier
 * features [sin(2 pi B c), cos(2 pi B c)] (B: 32 x 4, fixed), four SiLU
 * layers of width 64, one linear output. params: float32 vector of
 * NGG_MLP_NPARAM values laid out W1[64][64] b1[64] W2 b2 W3 b3 W4 b4 Wo[64]
 * bo B[32][4]; the first NGG_MLP_NTRAINED are trained. All pointers are
 * device pointers. z float32 (n, 3); y, target float32 (n).
 *
 * ngg_mlp_forward: y = net(z), FP32 on CUDA cores (the training precision).
 * ngg_mlp_forward_tc: the same network with the four 64x64 layers on the
 *   tcgen05 tensor cores (BF16 operands, FP32 accumulation in tensor memory);
 *   features and the output layer in FP32.
 * ngg_mlp_loss_grad: loss = mean((y - target)^2) (float64, device) and its
 *   gradient w.r.t. params (float32, NGG_MLP_NPARAM; zero for B).
 * ngg_mlp_adam: one bias-corrected Adam step (step >= 1) on the trained
 *   parameters; m, v float32 (NGG_MLP_NTRAINED).
 * ngg_mlp_train: n_steps Adam steps on random batches (batch rows drawn by a
 *   counter-based hash of (seed, step)) of the n_samples (z, target) pairs,
 *   learning rate cosine-decayed from lr0 to lr1; steps are numbered from
 *   step0 + 1; the loss of each step goes to loss_history (device float64,
 *   n_steps) when it is not NULL. */
typedef struct NggMlpScale {
    double x_scale, y_scale;    /* z_x = x * x_scale, z_y = y * y_scale (x, y table offsets) */
    double f_center, f_scale;   /* z_f = (f - f_center) * f_scale (Hz)                       */
    double out_scale;           /* table value = net output * out_scale                      */
} NggMlpScale;

#define NGG_MLP_NPARAM 16833
#define NGG_MLP_NTRAINED 16705
int ngg_mlp_forward(const float *params, const float *z, int64_t n, float *y, void *stream);
int ngg_mlp_forward_tc(const float *params, const float *z, int64_t n, float *y, void *stream);
int ngg_mlp_loss_grad(const float *params, const float *z, const float *target, int64_t n, float *grad,
                      double *loss, void *stream);
int ngg_mlp_adam(float *params, const float *grad, float *m, float *v, float lr, float beta1, float beta2,
                 float eps, int step, void *stream);
int ngg_mlp_train(float *params, float *m, float *v, const float *z, const float *target, int64_t n_samples,
                  int64_t batch, int n_steps, int step0, float lr0, float lr1, uint64_t seed,
                  double *loss_history, void *stream);

/* Mosaic gridding with the learned GCF in place of the table (the table path,
 * ngg_grid_gcf, stays the fallback and the yardstick for its error). Same
 * arguments as ngg_grid_gcf except: conv_kernel is not read; the GCF of
 * channel c is the network evaluated at freq[c] (one table per channel, so
 * n_cf_baseline = n_cf_pol = 1 and n_cf_chan = n_chan are required and the
 * CF maps are not read); support (n_chan, 2) int32 gives each channel's
 * support; conv_size = (max support + 1) * oversampling. The per-channel
 * tables are synthesised on the tensor cores (ngg_mlp_forward_tc's kernel)
 * for every tap and oversampling offset the gridder reads. */
int ngg_grid_gcf_learned(const NggGcfArgs *args, const float *params, const NggMlpScale *scale, void *stream);

/* ---- direction rotation (ngcasa/imaging/direction_rotate.py) ---------------
 * ngg_rotate_uvw replaces apply_rotation_matrix (:189-211) and the phase-
 * direction product of apply_phasor (:225-234): for every (time, baseline)
 * row, uvw_rot = uvw @ rotmat[f] (row vector times the 3x3 matrix of the
 * row's field f = row_field[time], an index into the n_field matrices) and
 * phase_dir = uvw_rot[0:k] . phase_rotation[f][0:k], k = 2 with common
 * tangent reprojection, else 3. uvw, uvw_rot (T,B,3) f64; rotmat (n_field,
 * 3,3) f64 (calc_rotation_mats, :127-173, computed on the host);
 * phase_rotation (n_field,3) f64; phase_dir (T,B) f64; row_field (T) int32. */
int ngg_rotate_uvw(const double *uvw, const int32_t *row_field, int64_t n_time, int64_t n_baseline,
                   const double *rotmat, const double *phase_rotation, int n_field,
                   int common_tangent_reprojection, double *uvw_rot, double *phase_dir, void *stream);

/* ngg_phase_rotate replaces the phasor of apply_phasor (:236-248):
 * vis_rot[t,b,c,p] = vis[t,b,c,p] * exp(2 pi i phase_dir[t,b] f[c] / c).
 * vis complex64 (T,B,C,P); freq_over_c (C) f64 = freq / 299792458;
 * single_precision != 0: vis_rot complex64 (the reference rounds its FP64
 * product to complex64); else complex128. */
int ngg_phase_rotate(const void *vis, const double *phase_dir, int64_t n_time, int64_t n_baseline,
                     int64_t n_chan, int64_t n_pol, const double *freq_over_c, int single_precision,
                     void *vis_rot, void *stream);

/* ---- Hogbom CLEAN minor cycle ------------------------------------------------
 * Replaces _clean_jit with _abs_image_peaks (ngcasa/deconvolution/
 * deconvolve_point_clean.py:174-236, 303-320), one call for all planes.
 * residual (n_planes, nx, ny) f64: the dirty planes in, the residuals out;
 * model (n_planes, nx, ny) f64: components added in place (zero it first);
 * psf (n_planes, px, py) f64, centre (px/2, py/2). Per plane: the peak is
 * the first pixel in scan order of largest |residual| (> 0, never NaN);
 * iterate while |peak| > threshold*|first peak| and fewer than n_iter
 * subtractions: model[peak] += gain*peak; residual -= s*psf shifted to the
 * peak over the overlap, s = gain*peak (scale_by_peak != 0, Hogbom's
 * algorithm) or s = gain (the reference's code as written). FP64 with the
 * reference's rounding: bit-identical results. iterations (n_planes) int32,
 * optional: subtractions done per plane. */
int ngg_hogbom_clean(double *residual, const double *psf, double *model, int64_t n_planes, int64_t nx,
                     int64_t ny, int64_t px, int64_t py, double gain, double threshold, int n_iter,
                     int scale_by_peak, int32_t *iterations, void *stream);

/* Profiling: when enabled, ngg_grid_ps records CUDA events on its stream
 * around its preparation phase (binning and the packing pass over the
 * visibilities) and its tile pass (the zeroing of split tiles and the tile
 * accumulation kernel). ngg_last_phase_ms waits for the last call's events
 * and returns the two durations (ms). */
void ngg_set_profiling(int enable);
int ngg_last_phase_ms(double *binning_ms, double *tiles_ms);

/* Release cached cuFFT plans and scratch held by the library. */
void ngg_release_cache(void);

#ifdef __cplusplus
}
#endif
#endif /* NGG_H */
