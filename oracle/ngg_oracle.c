/*
 * FP64 CPU restatement of the reference's standard gridder and imaging-weight
 * lookup.  TEST INFRASTRUCTURE: the checker for the CUDA path at sizes the
 * numpy oracle cannot reach, and the timed CPU baseline.  Never linked into
 * the product library.
 *
 * Restates, loop for loop:
 *   _standard_grid_jit           ngcasa/imaging/_imaging_utils/_standard_grid.py:242-371
 *   _standard_imaging_weight_degrid_jit                       _standard_grid.py:466-518
 * including the rounding rules int(pos+0.5) (truncation), floor(off*os+0.5),
 * the table index |os*i+off|, the whole-visibility edge rule and the NaN /
 * zero skips.  Cube mode runs channels in parallel (OpenMP); inside a channel
 * the addends reach every cell in the reference order (time, baseline, pol,
 * v-tap, u-tap), so results are bit-identical to the reference.  Continuum
 * mode splits the time axis into chunks gridded into private grids and adds
 * them with the pairwise tree of _tree_sum_list (_standard_grid.py:109-120),
 * as the reference's dask graph does for chunked input.
 *
 * Compile with -ffp-contract=off: the reference performs separate multiply
 * and add roundings.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define C_LIGHT 299792458.0

enum { MODE_DATA = 0, MODE_PSF = 1, MODE_DENSITY = 2 };

static void uv_scale(const double *freq, int n_chan, const double dl[2], const int64_t n_uv[2],
                     double *su, double *sv) {
    for (int c = 0; c < n_chan; ++c) {
        su[c] = -(freq[c] * dl[0] * (double)n_uv[0]) / C_LIGHT;
        sv[c] = -(freq[c] * dl[1] * (double)n_uv[1]) / C_LIGHT;
    }
}

/* grid one channel (or, for continuum chunks, a time range of all channels)
 * into grid (re/im interleaved complex128 when complex_grid, else double). */
static void grid_block(int mode, const float *vis, const double *uvw, const double *weight,
                       int64_t T0, int64_t T1, int64_t B, int64_t C, int64_t P,
                       int64_t c0, int64_t c1, int continuum,
                       const double *su, const double *sv, const double *cgk, int support,
                       int oversampling, const int64_t n_uv[2], double *grid, double *sumw) {
    const int sc = support / 2;
    const int64_t nu = n_uv[0], nv = n_uv[1];
    const int64_t ucen = nu / 2, vcen = nv / 2;
    const int cplx = (mode == MODE_DATA);
    const int64_t plane = nu * nv;
    for (int64_t t = T0; t < T1; ++t) {
        for (int64_t b = 0; b < B; ++b) {
            const double uw = uvw[(t * B + b) * 3 + 0];
            const double vw = uvw[(t * B + b) * 3 + 1];
            for (int64_t c = c0; c < c1; ++c) {
                const int64_t ac = continuum ? 0 : c;
                const double u = uw * su[c];
                const double v = vw * sv[c];
                if (isnan(u) || isnan(v)) continue;
                const double u_pos = u + (double)ucen;
                const double v_pos = v + (double)vcen;
                const double u_pos_c = -u + (double)ucen;
                const double v_pos_c = -v + (double)vcen;
                const double tu = trunc(u_pos + 0.5), tv = trunc(v_pos + 0.5);
                if (!(tu + sc < (double)nu && tv + sc < (double)nv && tu - sc >= 0 && tv - sc >= 0)) continue;
                const int64_t cu = (int64_t)tu, cv = (int64_t)tv;
                const int64_t cuc = (int64_t)trunc(u_pos_c + 0.5);
                const int64_t cvc = (int64_t)trunc(v_pos_c + 0.5);
                const int64_t ou = (int64_t)floor(((double)cu - u_pos) * oversampling + 0.5);
                const int64_t ov = (int64_t)floor(((double)cv - v_pos) * oversampling + 0.5);
                double conv_u[64], conv_v[64];
                for (int i = -sc; i < support - sc; ++i) {
                    conv_u[i + sc] = cgk[llabs((int64_t)oversampling * i + ou)];
                    conv_v[i + sc] = cgk[llabs((int64_t)oversampling * i + ov)];
                }
                const int64_t row = ((t * B + b) * C + c) * P;
                for (int64_t p = 0; p < P; ++p) {
                    double wr, wi = 0.0, selw;
                    const double w = weight[row + p];
                    if (mode == MODE_DATA) {
                        const double vr = (double)vis[2 * (row + p)], vi = (double)vis[2 * (row + p) + 1];
                        wr = vr * w;
                        wi = vi * w;
                        selw = w;
                        if (isnan(wr) || isnan(wi) || (wr == 0.0 && wi == 0.0)) continue;
                    } else {
                        if (mode == MODE_DENSITY && P >= 2) {
                            wr = (weight[row + 0] + weight[row + 1]) / 2.0;
                        } else {
                            wr = w;
                        }
                        selw = wr;
                        if (isnan(wr) || wr == 0.0) continue;
                    }
                    double *gp = grid + (ac * P + p) * plane * (cplx ? 2 : 1);
                    double norm = 0.0;
                    for (int iv = -sc; iv < support - sc; ++iv) {
                        const double cvv = conv_v[iv + sc];
                        const int64_t vi_ = cv + iv;
                        const int64_t vic = cvc + iv;
                        for (int iu = -sc; iu < support - sc; ++iu) {
                            const double conv = conv_u[iu + sc] * cvv;
                            const int64_t ui_ = cu + iu;
                            if (cplx) {
                                gp[2 * (ui_ * nv + vi_)] += conv * wr;
                                gp[2 * (ui_ * nv + vi_) + 1] += conv * wi;
                            } else {
                                gp[ui_ * nv + vi_] += conv * wr;
                            }
                            norm = norm + conv;
                            if (mode == MODE_DENSITY) {
                                const int64_t uic = cuc + iu;
                                /* the reference does not bound-check the mirrored
                                 * cell; it is only off the grid for cells on the
                                 * last two rows/columns of the edge */
                                if (uic >= 0 && uic < nu && vic >= 0 && vic < nv)
                                    gp[uic * nv + vic] += conv * wr;
                            }
                        }
                    }
                    sumw[ac * P + p] += selw * norm;
                    if (mode == MODE_DENSITY) sumw[ac * P + p] += selw * norm;
                }
            }
        }
    }
}

/* Returns 0 on success, -1 on bad arguments / allocation failure. */
int ngg_oracle_grid(int mode, const float *vis, const double *uvw, const double *weight,
                    int64_t T, int64_t B, int64_t C, int64_t P, const double *freq,
                    const double *cgk, int support, int oversampling, const int64_t n_uv[2],
                    const double dl[2], int continuum, int n_threads, double *grid, double *sumw) {
    if (T < 0 || B < 0 || C < 0 || P < 0 || support < 1 || support > 63) return -1;
    if (mode == MODE_DATA && !vis) return -1;
    double *su = (double *)malloc(sizeof(double) * (C > 0 ? C : 1));
    double *sv = (double *)malloc(sizeof(double) * (C > 0 ? C : 1));
    if (!su || !sv) { free(su); free(sv); return -1; }
    uv_scale(freq, (int)C, dl, n_uv, su, sv);
    const int cplx = (mode == MODE_DATA);
    const int64_t n_img = continuum ? 1 : C;
    const size_t plane = (size_t)n_uv[0] * (size_t)n_uv[1] * (cplx ? 2 : 1);
    memset(grid, 0, sizeof(double) * plane * (size_t)(n_img * P));
    memset(sumw, 0, sizeof(double) * (size_t)(n_img * P));
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
    if (!continuum) {
#pragma omp parallel for schedule(dynamic, 1)
        for (int64_t c = 0; c < C; ++c)
            grid_block(mode, vis, uvw, weight, 0, T, B, C, P, c, c + 1, 0, su, sv, cgk, support,
                       oversampling, n_uv, grid, sumw);
    } else {
        int nchunk = 1;
#ifdef _OPENMP
        nchunk = n_threads > 0 ? n_threads : omp_get_max_threads();
#endif
        if (nchunk > T) nchunk = T > 0 ? (int)T : 1;
        if (nchunk <= 1) {
            grid_block(mode, vis, uvw, weight, 0, T, B, C, P, 0, C, 1, su, sv, cgk, support,
                       oversampling, n_uv, grid, sumw);
        } else {
            const size_t gsz = plane * (size_t)P;
            double **pg = (double **)calloc(nchunk, sizeof(double *));
            double **ps = (double **)calloc(nchunk, sizeof(double *));
            int bad = !pg || !ps;
            for (int k = 0; !bad && k < nchunk; ++k) {
                pg[k] = k == 0 ? grid : (double *)calloc(gsz, sizeof(double));
                ps[k] = k == 0 ? sumw : (double *)calloc((size_t)P, sizeof(double));
                if (!pg[k] || !ps[k]) bad = 1;
            }
            if (!bad) {
#pragma omp parallel for schedule(static, 1)
                for (int k = 0; k < nchunk; ++k) {
                    const int64_t t0 = T * k / nchunk, t1 = T * (k + 1) / nchunk;
                    grid_block(mode, vis, uvw, weight, t0, t1, B, C, P, 0, C, 1, su, sv, cgk,
                               support, oversampling, n_uv, pg[k], ps[k]);
                }
                /* pairwise tree, as _tree_sum_list */
                for (int step = 1; step < nchunk; step *= 2) {
#pragma omp parallel for schedule(static, 1)
                    for (int k = 0; k < nchunk; k += 2 * step) {
                        if (k + step < nchunk) {
                            for (size_t i = 0; i < gsz; ++i) pg[k][i] += pg[k + step][i];
                            for (int64_t p = 0; p < P; ++p) ps[k][p] += ps[k + step][p];
                        }
                    }
                }
            }
            for (int k = 1; pg && ps && k < nchunk; ++k) { free(pg[k]); free(ps[k]); }
            free(pg); free(ps);
            if (bad) { free(su); free(sv); return -1; }
        }
    }
    free(su);
    free(sv);
    return 0;
}

/* _standard_imaging_weight_degrid_jit; density is (u,v,Cimg,P) float64. */
int ngg_oracle_weight_degrid(const double *density, const double *uvw, const double *weight,
                             const double *briggs, int64_t T, int64_t B, int64_t C, int64_t P,
                             const double *freq, const int64_t n_uv[2], const double dl[2],
                             int continuum, int n_threads, double *out) {
    double *su = (double *)malloc(sizeof(double) * (C > 0 ? C : 1));
    double *sv = (double *)malloc(sizeof(double) * (C > 0 ? C : 1));
    if (!su || !sv) { free(su); free(sv); return -1; }
    uv_scale(freq, (int)C, dl, n_uv, su, sv);
    const int64_t n_img = continuum ? 1 : C;
    const int64_t nu = n_uv[0], nv = n_uv[1];
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < T; ++t) {
        for (int64_t b = 0; b < B; ++b) {
            for (int64_t c = 0; c < C; ++c) {
                const int64_t ac = continuum ? 0 : c;
                const int64_t row = ((t * B + b) * C + c) * P;
                for (int64_t p = 0; p < P; ++p) out[row + p] = 0.0;
                const double u = uvw[(t * B + b) * 3 + 0] * su[c];
                const double v = uvw[(t * B + b) * 3 + 1] * sv[c];
                if (isnan(u) || isnan(v)) continue;
                const double tu = trunc(u + (double)(nu / 2) + 0.5);
                const double tv = trunc(v + (double)(nv / 2) + 0.5);
                if (!(tu < (double)nu && tv < (double)nv && tu >= 0 && tv >= 0)) continue;
                const int64_t cu = (int64_t)tu, cv = (int64_t)tv;
                for (int64_t p = 0; p < P; ++p) {
                    double iw = (P == 2) ? (weight[row + 0] + weight[row + 1]) / 2.0 : weight[row + p];
                    const double wp = weight[row + p];
                    const double W = density[((cu * nv + cv) * n_img + ac) * P + p];
                    if (!isnan(wp) && wp != 0.0 && !isnan(W) && W != 0.0)
                        iw = iw / (briggs[(0 * n_img + ac) * P + p] * W + briggs[(1 * n_img + ac) * P + p]);
                    out[row + p] = iw;
                }
            }
        }
    }
    free(su);
    free(sv);
    return 0;
}

/* ------------------------------------------------------------------------
 * Mosaic gridders, restating loop for loop
 *   _aperture_grid_jit          ngcasa/imaging/_imaging_utils/_aperture_grid.py:376-513
 *   _aperture_weight_grid_jit   _aperture_grid.py:180-291
 * conv = table[cfb,cfc,cfp,x,y] * phase_gradient[field,x,y] evaluated as
 * (k*pr, k*pi); addend = conv * weighted_data with the scalar complex
 * formula; norm summed in tap order; sum_weight += w*Re(norm^2) (data) or
 * w*Re(norm) (psf, weight).  Cube mode runs channels in parallel (each
 * channel's cells and sums receive their addends in the reference order);
 * continuum mode is sequential.
 *   kind: 0 data, 1 psf, 2 weight grid (taps at the grid centre, zero offset)
 *   field_index (T,B): index into the phase-gradient planes, < 0 skips the row
 *   table (ncfb,ncfc,ncfp,R0,R1) f64; support (ncfb,ncfc,ncfp,2) int64;
 *   pg (n_field,R0,R1) complex128; grid complex128 (Cimg,P,Nu,Nv).
 * ------------------------------------------------------------------------ */
static void aperture_block(int kind, const float *vis, const double *uvw, const double *weight,
                           const int64_t *field_index, int64_t T, int64_t B, int64_t C, int64_t P,
                           int64_t c0, int64_t c1, int continuum, const double *su, const double *sv,
                           const int64_t *cfb_map, const int64_t *cfc_map, const int64_t *cfp_map,
                           int64_t ncfc, int64_t ncfp, const double *table, const int64_t *support,
                           int64_t maxsup, const double *pg, int64_t R0, int64_t R1, const int64_t os[2],
                           const int64_t n_uv[2], double *grid, double *sumw) {
    const int64_t nu = n_uv[0], nv = n_uv[1], ucen = nu / 2, vcen = nv / 2;
    const int64_t cc0 = R0 / 2, cc1 = R1 / 2;
    for (int64_t t = 0; t < T; ++t) {
        for (int64_t b = 0; b < B; ++b) {
            const int64_t fi = field_index[t * B + b];
            if (fi < 0) continue;
            const int64_t cfb = cfb_map[b];
            for (int64_t c = c0; c < c1; ++c) {
                const int64_t cfc = cfc_map[c];
                const int64_t ac = continuum ? 0 : c;
                const double u = uvw[(t * B + b) * 3 + 0] * su[c];
                const double v = uvw[(t * B + b) * 3 + 1] * sv[c];
                if (isnan(u) || isnan(v)) continue;
                const double up = u + (double)ucen, vp = v + (double)vcen;
                const int64_t cu = (int64_t)(up + 0.5), cv = (int64_t)(vp + 0.5);
                if (!(cu + maxsup < nu && cv + maxsup < nv && cu - maxsup >= 0 && cv - maxsup >= 0)) continue;
                int64_t ou, ov, gu, gv;
                if (kind == 2) {
                    ou = cc0; ov = cc1; gu = ucen; gv = vcen;
                } else {
                    ou = (int64_t)floor(((double)cu - up) * (double)os[0] + 0.5) + cc0;
                    ov = (int64_t)floor(((double)cv - vp) * (double)os[1] + 0.5) + cc1;
                    gu = cu; gv = cv;
                }
                for (int64_t p = 0; p < P; ++p) {
                    const int64_t vi = ((t * B + b) * C + c) * P + p;
                    const double w = weight[vi];
                    double wr, wi;
                    if (kind == 0) {
                        wr = (double)vis[2 * vi] * w;
                        wi = (double)vis[2 * vi + 1] * w;
                        if (isnan(wr) || isnan(wi) || (wr == 0.0 && wi == 0.0)) continue;
                    } else {
                        wr = w; wi = 0.0;
                        if (isnan(w) || w == 0.0) continue;
                    }
                    const int64_t cfp = cfp_map[p];
                    const int64_t cf = (cfb * ncfc + cfc) * ncfp + cfp;
                    const int64_t s_u = support[cf * 2], s_v = support[cf * 2 + 1];
                    double nr = 0.0, ni = 0.0;
                    double *g = grid + 2 * ((ac * P + p) * nu * nv);
                    for (int64_t iv = -(s_v / 2); iv < s_v - s_v / 2; ++iv) {
                        const int64_t y = os[1] * iv + ov;
                        for (int64_t iu = -(s_u / 2); iu < s_u - s_u / 2; ++iu) {
                            const int64_t x = os[0] * iu + ou;
                            const double k = table[(cf * R0 + x) * R1 + y];
                            const double *ph = pg + 2 * ((fi * R0 + x) * R1 + y);
                            const double cr = k * ph[0], ci = k * ph[1];
                            const double ar = cr * wr - ci * wi, ai = cr * wi + ci * wr;
                            double *cell = g + 2 * ((gu + iu) * nv + (gv + iv));
                            cell[0] = cell[0] + ar;
                            cell[1] = cell[1] + ai;
                            nr = nr + cr;
                            ni = ni + ci;
                        }
                    }
                    double *s = sumw + ac * P + p;
                    if (kind == 0) *s = *s + w * (nr * nr - ni * ni);
                    else *s = *s + w * nr;
                }
            }
        }
    }
}

int ngg_oracle_aperture_grid(int kind, const float *vis, const double *uvw, const double *weight,
                             const int64_t *field_index, int64_t T, int64_t B, int64_t C, int64_t P,
                             const double *freq, const int64_t *cfb_map, const int64_t *cfc_map,
                             const int64_t *cfp_map, int64_t ncfb, int64_t ncfc, int64_t ncfp,
                             const double *table, const int64_t *support, const double *pg, int64_t n_field,
                             int64_t R0, int64_t R1, const int64_t os[2], const int64_t n_uv[2],
                             const double dl[2], int continuum, int n_threads, double *grid, double *sumw) {
    (void)ncfb; (void)n_field;
    const int64_t n_img = continuum ? 1 : C;
    memset(grid, 0, sizeof(double) * 2 * (size_t)(n_img * P * n_uv[0] * n_uv[1]));
    memset(sumw, 0, sizeof(double) * (size_t)(n_img * P));
    if (T * B * C == 0) return 0;
    double *su = malloc(sizeof(double) * C), *sv = malloc(sizeof(double) * C);
    if (!su || !sv) { free(su); free(sv); return 1; }
    uv_scale(freq, (int)C, dl, n_uv, su, sv);
    int64_t maxsup = 0;
    for (int64_t i = 0; i < ncfb * ncfc * ncfp * 2; ++i) maxsup = support[i] > maxsup ? support[i] : maxsup;
    if (continuum) {
        aperture_block(kind, vis, uvw, weight, field_index, T, B, C, P, 0, C, 1, su, sv, cfb_map, cfc_map, cfp_map,
                       ncfc, ncfp, table, support, maxsup, pg, R0, R1, os, n_uv, grid, sumw);
    } else {
#ifdef _OPENMP
        if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
        for (int64_t c = 0; c < C; ++c)
            aperture_block(kind, vis, uvw, weight, field_index, T, B, C, P, c, c + 1, 0, su, sv, cfb_map, cfc_map,
                           cfp_map, ncfc, ncfp, table, support, maxsup, pg, R0, R1, os, n_uv, grid, sumw);
    }
    free(su);
    free(sv);
    return 0;
}
