/*
 * CPU oracle for the W-projection gridding path -- TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C, the serial algorithm of the reference
 * gridder so that the CUDA library can be checked against it.  Only the test
 * suite, the smoke check and the CPU-baseline leg of the benchmark load it;
 * the product library never links or calls it.
 *
 * Parity is pinned two ways: the restatement is checked bit-for-bit against
 * the reference function compiled from its own source (oracle/_ref, built by
 * oracle/Makefile where the reference tree is present), and against golden
 * vectors produced by that compiled reference and committed under
 * tests/golden/.
 *
 * Reference files cited (paths within the reference project):
 *   oskar_grid_wproj.c:37-123    oskar_grid_wproj_d  (FP64 gridder)
 *   oskar_grid_wproj.c:126-212   oskar_grid_wproj_f  (FP32 gridder, FP64 norm)
 *   utils/oskar_grid_weights.c:38-172  uniform-weighting density write/read
 *
 * Build with -ffp-contract=off: the reference is compiled for baseline
 * x86-64, which has no fused multiply-add, so no contraction may happen on an
 * FMA-capable host (aarch64) either, or FP32 bit-parity is lost.
 */
#include <math.h>
#include <pthread.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#if defined(__GNUC__)
#define ORACLE_API __attribute__((visibility("default")))
#else
#define ORACLE_API
#endif

/* ------------------------------------------------------------------------ */
/* Placement                                                                */
/* ------------------------------------------------------------------------ */

typedef struct
{
    int gu, gv;     /* grid cell of the visibility centre */
    int ou, ov;     /* oversampled offset from the cell centre */
    int plane;      /* w-plane after the clamp to the last plane */
    int conj_neg;   /* 1 when the kernel's imaginary part is negated (ww > 0) */
    int support;    /* support of that plane */
    int skipped;    /* 1 when the footprint leaves the grid */
} oracle_place_t;

/* Placement of one FP32 visibility in the order oskar_grid_wproj.c:146-187
 * evaluates it: cell = round(pos) + centre, offset = round((round(pos) - pos)
 * * oversample), plane = round(sqrt(|ww * w_scale|)) clamped to the last
 * plane, skip when any edge of the (2 support + 1)^2 footprint leaves
 * [0, grid_size). */
static oracle_place_t place_f(float uu, float vv, float ww, float grid_scale,
        int grid_centre, int grid_size, int oversample, size_t num_w_planes,
        const int* support, float w_scale)
{
    oracle_place_t p;
    const float pos_u = -uu * grid_scale;
    const float pos_v = vv * grid_scale;
    const size_t grid_w = (size_t)roundf(sqrtf(fabsf(ww * w_scale)));
    const float rpos_u = roundf(pos_u), rpos_v = roundf(pos_v);
    p.conj_neg = (ww > 0.0f);
    p.gu = (int)rpos_u + grid_centre;
    p.gv = (int)rpos_v + grid_centre;
    p.ou = (int)roundf((rpos_u - pos_u) * oversample);
    p.ov = (int)roundf((rpos_v - pos_v) * oversample);
    p.plane = grid_w < num_w_planes ? (int)grid_w : (int)num_w_planes - 1;
    p.support = support[p.plane];
    p.skipped = (p.gu + p.support >= grid_size || p.gu - p.support < 0 ||
            p.gv + p.support >= grid_size || p.gv - p.support < 0);
    return p;
}

/* FP64 placement, oskar_grid_wproj.c:57-98. */
static oracle_place_t place_d(double uu, double vv, double ww,
        double grid_scale, int grid_centre, int grid_size, int oversample,
        size_t num_w_planes, const int* support, double w_scale)
{
    oracle_place_t p;
    const double pos_u = -uu * grid_scale;
    const double pos_v = vv * grid_scale;
    const size_t grid_w = (size_t)round(sqrt(fabs(ww * w_scale)));
    const double rpos_u = round(pos_u), rpos_v = round(pos_v);
    p.conj_neg = (ww > 0.0);
    p.gu = (int)rpos_u + grid_centre;
    p.gv = (int)rpos_v + grid_centre;
    p.ou = (int)round((rpos_u - pos_u) * oversample);
    p.ov = (int)round((rpos_v - pos_v) * oversample);
    p.plane = grid_w < num_w_planes ? (int)grid_w : (int)num_w_planes - 1;
    p.support = support[p.plane];
    p.skipped = (p.gu + p.support >= grid_size || p.gu - p.support < 0 ||
            p.gv + p.support >= grid_size || p.gv - p.support < 0);
    return p;
}

/* Per-visibility placement, FP32 rules.  Arrays of length num_points;
 * returns the number of skipped visibilities. */
ORACLE_API size_t oracle_place_f(size_t num_w_planes, const int* support,
        int oversample, size_t num_points, const float* uu, const float* vv,
        const float* ww, float cell_size_rad, float w_scale, int grid_size,
        int* gu, int* gv, int* ou, int* ov, int* plane, int* conj_neg,
        int* skipped)
{
    size_t i, n_skip = 0;
    const int centre = grid_size / 2;
    const float scale = grid_size * cell_size_rad;
    for (i = 0; i < num_points; ++i)
    {
        oracle_place_t p = place_f(uu[i], vv[i], ww[i], scale, centre,
                grid_size, oversample, num_w_planes, support, w_scale);
        gu[i] = p.gu; gv[i] = p.gv; ou[i] = p.ou; ov[i] = p.ov;
        plane[i] = p.plane; conj_neg[i] = p.conj_neg; skipped[i] = p.skipped;
        n_skip += (size_t)p.skipped;
    }
    return n_skip;
}

/* Per-visibility placement, FP64 rules. */
ORACLE_API size_t oracle_place_d(size_t num_w_planes, const int* support,
        int oversample, size_t num_points, const double* uu, const double* vv,
        const double* ww, double cell_size_rad, double w_scale, int grid_size,
        int* gu, int* gv, int* ou, int* ov, int* plane, int* conj_neg,
        int* skipped)
{
    size_t i, n_skip = 0;
    const int centre = grid_size / 2;
    const double scale = grid_size * cell_size_rad;
    for (i = 0; i < num_points; ++i)
    {
        oracle_place_t p = place_d(uu[i], vv[i], ww[i], scale, centre,
                grid_size, oversample, num_w_planes, support, w_scale);
        gu[i] = p.gu; gv[i] = p.gv; ou[i] = p.ou; ov[i] = p.ov;
        plane[i] = p.plane; conj_neg[i] = p.conj_neg; skipped[i] = p.skipped;
        n_skip += (size_t)p.skipped;
    }
    return n_skip;
}

/* ------------------------------------------------------------------------ */
/* Serial gridders (the contract)                                           */
/* ------------------------------------------------------------------------ */

/* Restatement of oskar_grid_wproj_f, oskar_grid_wproj.c:126-212.  The cell
 * update is evaluated exactly as the reference does: the product difference
 * is formed in FP32 and then added to the cell; the tap sum is FP64 over the
 * real parts in (j outer, k inner) order. */
ORACLE_API void oracle_grid_wproj_f(size_t num_w_planes, const int* support,
        int oversample, int conv_size_half, const float* conv_func,
        size_t num_points, const float* uu, const float* vv, const float* ww,
        const float* vis, const float* weight, float cell_size_rad,
        float w_scale, int grid_size, size_t* num_skipped, double* norm,
        float* grid)
{
    size_t i, n_skip = 0;
    const size_t plane_stride = (size_t)(conv_size_half * conv_size_half);
    const int centre = grid_size / 2;
    const float scale = grid_size * cell_size_rad;
    for (i = 0; i < num_points; ++i)
    {
        int j, k;
        double tap_sum = 0.0;
        const oracle_place_t p = place_f(uu[i], vv[i], ww[i], scale, centre,
                grid_size, oversample, num_w_planes, support, w_scale);
        const float conj = p.conj_neg ? -1.0f : 1.0f;
        const float w_i = weight[i];
        const float v_re = w_i * vis[2 * i];
        const float v_im = w_i * vis[2 * i + 1];
        const size_t kstart = (size_t)p.plane * plane_stride;
        const int s = p.support;
        if (p.skipped) { n_skip++; continue; }
        for (j = -s; j <= s; ++j)
        {
            const size_t row = (size_t)(p.gv + j) * (size_t)grid_size +
                    (size_t)p.gu;
            const size_t krow = kstart +
                    (size_t)abs(p.ov + j * oversample) * conv_size_half;
            for (k = -s; k <= s; ++k)
            {
                const size_t t = (krow + abs(p.ou + k * oversample)) << 1;
                const size_t c = (row + k) << 1;
                const float c_re = conv_func[t];
                const float c_im = conv_func[t + 1] * conj;
                grid[c]     += (v_re * c_re - v_im * c_im);
                grid[c + 1] += (v_im * c_re + v_re * c_im);
                tap_sum += c_re;
            }
        }
        *norm += tap_sum * w_i;
    }
    *num_skipped = n_skip;
}

/* Restatement of oskar_grid_wproj_d, oskar_grid_wproj.c:37-123. */
ORACLE_API void oracle_grid_wproj_d(size_t num_w_planes, const int* support,
        int oversample, int conv_size_half, const double* conv_func,
        size_t num_points, const double* uu, const double* vv,
        const double* ww, const double* vis, const double* weight,
        double cell_size_rad, double w_scale, int grid_size,
        size_t* num_skipped, double* norm, double* grid)
{
    size_t i, n_skip = 0;
    const size_t plane_stride = (size_t)(conv_size_half * conv_size_half);
    const int centre = grid_size / 2;
    const double scale = grid_size * cell_size_rad;
    for (i = 0; i < num_points; ++i)
    {
        int j, k;
        double tap_sum = 0.0;
        const oracle_place_t p = place_d(uu[i], vv[i], ww[i], scale, centre,
                grid_size, oversample, num_w_planes, support, w_scale);
        const double conj = p.conj_neg ? -1.0 : 1.0;
        const double w_i = weight[i];
        const double v_re = w_i * vis[2 * i];
        const double v_im = w_i * vis[2 * i + 1];
        const size_t kstart = (size_t)p.plane * plane_stride;
        const int s = p.support;
        if (p.skipped) { n_skip++; continue; }
        for (j = -s; j <= s; ++j)
        {
            const size_t row = (size_t)(p.gv + j) * (size_t)grid_size +
                    (size_t)p.gu;
            const size_t krow = kstart +
                    (size_t)abs(p.ov + j * oversample) * conv_size_half;
            for (k = -s; k <= s; ++k)
            {
                const size_t t = (krow + abs(p.ou + k * oversample)) << 1;
                const size_t c = (row + k) << 1;
                const double c_re = conv_func[t];
                const double c_im = conv_func[t + 1] * conj;
                grid[c]     += (v_re * c_re - v_im * c_im);
                grid[c + 1] += (v_im * c_re + v_re * c_im);
                tap_sum += c_re;
            }
        }
        *norm += tap_sum * w_i;
    }
    *num_skipped = n_skip;
}

/* ------------------------------------------------------------------------ */
/* FP64 reference answer for FP32 inputs                                    */
/* ------------------------------------------------------------------------ */

/* The oskar_grid_wproj_d accumulation (oskar_grid_wproj.c:100-121) applied
 * to FP32 inputs promoted to FP64, with the FP32 placement of
 * oskar_grid_wproj.c:146-187.  This is the error yardstick for the FP32 GPU
 * path: same cells, planes and offsets as the FP32 contract, no rounding in
 * the accumulation.  grid is FP64 complex (in/out). */
ORACLE_API void oracle_grid_wproj_f_fp64acc(size_t num_w_planes,
        const int* support, int oversample, int conv_size_half,
        const float* conv_func, size_t num_points, const float* uu,
        const float* vv, const float* ww, const float* vis,
        const float* weight, float cell_size_rad, float w_scale,
        int grid_size, size_t* num_skipped, double* norm, double* grid)
{
    size_t i, n_skip = 0;
    const size_t plane_stride = (size_t)(conv_size_half * conv_size_half);
    const int centre = grid_size / 2;
    const float scale = grid_size * cell_size_rad;
    for (i = 0; i < num_points; ++i)
    {
        int j, k;
        double tap_sum = 0.0;
        const oracle_place_t p = place_f(uu[i], vv[i], ww[i], scale, centre,
                grid_size, oversample, num_w_planes, support, w_scale);
        const double conj = p.conj_neg ? -1.0 : 1.0;
        const double w_i = weight[i];
        const double v_re = w_i * (double)vis[2 * i];
        const double v_im = w_i * (double)vis[2 * i + 1];
        const size_t kstart = (size_t)p.plane * plane_stride;
        const int s = p.support;
        if (p.skipped) { n_skip++; continue; }
        for (j = -s; j <= s; ++j)
        {
            const size_t row = (size_t)(p.gv + j) * (size_t)grid_size +
                    (size_t)p.gu;
            const size_t krow = kstart +
                    (size_t)abs(p.ov + j * oversample) * conv_size_half;
            for (k = -s; k <= s; ++k)
            {
                const size_t t = (krow + abs(p.ou + k * oversample)) << 1;
                const size_t c = (row + k) << 1;
                const double c_re = conv_func[t];
                const double c_im = (double)conv_func[t + 1] * conj;
                grid[c]     += (v_re * c_re - v_im * c_im);
                grid[c + 1] += (v_im * c_re + v_re * c_im);
                tap_sum += c_re;
            }
        }
        *norm += tap_sum * w_i;
    }
    *num_skipped = n_skip;
}

/* ------------------------------------------------------------------------ */
/* Adjoint of the gridding map (degridding)                                 */
/* ------------------------------------------------------------------------ */

/* Exact adjoint, in FP64, of the complex-linear map v -> grid that
 * oskar_grid_wproj_f applies to the weighted visibilities v_i = w_i vis_i
 * (oskar_grid_wproj.c:190-209): out_i = sum over the footprint of
 * conj(c~_i(cell)) * grid(cell), where c~ is the tap with its imaginary part
 * negated for ww > 0.  Placement follows the FP32 rules; skipped
 * visibilities get 0.  The reference has no degridder; this definition is
 * pinned by the dot-product identity <G x, y> = <x, G^H y>. */
ORACLE_API void oracle_degrid_wproj_f_fp64(size_t num_w_planes,
        const int* support, int oversample, int conv_size_half,
        const float* conv_func, size_t num_points, const float* uu,
        const float* vv, const float* ww, float cell_size_rad,
        float w_scale, int grid_size, const double* grid, double* out_vis)
{
    size_t i;
    const size_t plane_stride = (size_t)(conv_size_half * conv_size_half);
    const int centre = grid_size / 2;
    const float scale = grid_size * cell_size_rad;
    for (i = 0; i < num_points; ++i)
    {
        int j, k;
        double acc_re = 0.0, acc_im = 0.0;
        const oracle_place_t p = place_f(uu[i], vv[i], ww[i], scale, centre,
                grid_size, oversample, num_w_planes, support, w_scale);
        const double conj = p.conj_neg ? -1.0 : 1.0;
        const size_t kstart = (size_t)p.plane * plane_stride;
        const int s = p.support;
        if (!p.skipped)
        {
            for (j = -s; j <= s; ++j)
            {
                const size_t row = (size_t)(p.gv + j) * (size_t)grid_size +
                        (size_t)p.gu;
                const size_t krow = kstart +
                        (size_t)abs(p.ov + j * oversample) * conv_size_half;
                for (k = -s; k <= s; ++k)
                {
                    const size_t t = (krow + abs(p.ou + k * oversample)) << 1;
                    const size_t c = (row + k) << 1;
                    const double c_re = conv_func[t];
                    const double c_im = (double)conv_func[t + 1] * conj;
                    const double g_re = grid[c], g_im = grid[c + 1];
                    /* conj(c) * g */
                    acc_re += c_re * g_re + c_im * g_im;
                    acc_im += c_re * g_im - c_im * g_re;
                }
            }
        }
        out_vis[2 * i] = acc_re;
        out_vis[2 * i + 1] = acc_im;
    }
}

/* The same adjoint for oskar_grid_wproj_d: FP64 placement rules and an FP64
 * kernel cube (oskar_grid_wproj.c:114-131 declares the _d variant). */
ORACLE_API void oracle_degrid_wproj_d(size_t num_w_planes,
        const int* support, int oversample, int conv_size_half,
        const double* conv_func, size_t num_points, const double* uu,
        const double* vv, const double* ww, double cell_size_rad,
        double w_scale, int grid_size, const double* grid, double* out_vis)
{
    size_t i;
    const size_t plane_stride = (size_t)(conv_size_half * conv_size_half);
    const int centre = grid_size / 2;
    const double scale = grid_size * cell_size_rad;
    for (i = 0; i < num_points; ++i)
    {
        int j, k;
        double acc_re = 0.0, acc_im = 0.0;
        const oracle_place_t p = place_d(uu[i], vv[i], ww[i], scale, centre,
                grid_size, oversample, num_w_planes, support, w_scale);
        const double conj = p.conj_neg ? -1.0 : 1.0;
        const size_t kstart = (size_t)p.plane * plane_stride;
        const int s = p.support;
        if (!p.skipped)
        {
            for (j = -s; j <= s; ++j)
            {
                const size_t row = (size_t)(p.gv + j) * (size_t)grid_size +
                        (size_t)p.gu;
                const size_t krow = kstart +
                        (size_t)abs(p.ov + j * oversample) * conv_size_half;
                for (k = -s; k <= s; ++k)
                {
                    const size_t t = (krow + abs(p.ou + k * oversample)) << 1;
                    const size_t c = (row + k) << 1;
                    const double c_re = conv_func[t];
                    const double c_im = conv_func[t + 1] * conj;
                    const double g_re = grid[c], g_im = grid[c + 1];
                    acc_re += c_re * g_re + c_im * g_im;
                    acc_im += c_re * g_im - c_im * g_re;
                }
            }
        }
        out_vis[2 * i] = acc_re;
        out_vis[2 * i + 1] = acc_im;
    }
}

/* ------------------------------------------------------------------------ */
/* Multi-threaded restatement of oskar_grid_wproj_f                         */
/* ------------------------------------------------------------------------ */

/* The CPU baseline on a many-core host.  Grid rows are split into bands and
 * each band is owned by one thread that walks all visibilities in input
 * order, so every cell receives its contributions in exactly the serial
 * order: the result is bit-identical to oracle_grid_wproj_f.  The tap sums
 * for the norm are formed per visibility in the serial (j, k) order and
 * accumulated into norm in input order, so norm is bit-identical too. */

typedef struct
{
    const float* conv_func;
    const float* vis;
    const float* weight;
    const oracle_place_t* place;
    float* grid;
    double* tap_sum;
    size_t num_points, plane_stride;
    int oversample, conv_size_half, grid_size, num_bands;
    const float* uu; const float* vv; const float* ww;
    const int* support;
    size_t num_w_planes;
    float cell_size_rad, w_scale;
    double* grid64;     /* non-null: FP64 accumulation into this grid */
    int place64;        /* 1: FP64 placement of the promoted coordinates */
    int next;           /* work counter, atomically incremented */
    int phase;          /* 0: placement + tap sums, 1: gridding bands */
    size_t chunk;
} mt_job_t;

static void mt_place_chunk(mt_job_t* job, size_t i0, size_t i1)
{
    size_t i;
    const int centre = job->grid_size / 2;
    const float scale = job->grid_size * job->cell_size_rad;
    /* oskar_grid_wproj.c:59: the FP64 grid scale of the promoted cell. */
    const double scale64 = job->grid_size * (double)job->cell_size_rad;
    for (i = i0; i < i1; ++i)
    {
        int j, k;
        double tap_sum = 0.0;
        const oracle_place_t p = job->place64 ?
                place_d((double)job->uu[i], (double)job->vv[i],
                        (double)job->ww[i], scale64, centre, job->grid_size,
                        job->oversample, job->num_w_planes, job->support,
                        (double)job->w_scale) :
                place_f(job->uu[i], job->vv[i], job->ww[i],
                        scale, centre, job->grid_size, job->oversample,
                        job->num_w_planes, job->support, job->w_scale);
        ((oracle_place_t*)job->place)[i] = p;
        if (!p.skipped)
        {
            const size_t kstart = (size_t)p.plane * job->plane_stride;
            for (j = -p.support; j <= p.support; ++j)
            {
                const size_t krow = kstart + (size_t)abs(p.ov +
                        j * job->oversample) * job->conv_size_half;
                for (k = -p.support; k <= p.support; ++k)
                    tap_sum += job->conv_func[
                            (krow + abs(p.ou + k * job->oversample)) << 1];
            }
        }
        job->tap_sum[i] = tap_sum;
    }
}

static void mt_grid_band(mt_job_t* job, int band)
{
    size_t i;
    const int G = job->grid_size;
    const int r0 = (int)(((long long)G * band) / job->num_bands);
    const int r1 = (int)(((long long)G * (band + 1)) / job->num_bands);
    const int os = job->oversample;
    for (i = 0; i < job->num_points; ++i)
    {
        int j, k, j0, j1;
        const oracle_place_t* p = &job->place[i];
        if (p->skipped) continue;
        j0 = r0 - p->gv; if (j0 < -p->support) j0 = -p->support;
        j1 = r1 - 1 - p->gv; if (j1 > p->support) j1 = p->support;
        if (j0 > j1) continue;
        if (job->grid64)
        {
            /* Same accumulation as oracle_grid_wproj_f_fp64acc. */
            const double conj = p->conj_neg ? -1.0 : 1.0;
            const double w_i = job->weight[i];
            const double v_re = w_i * (double)job->vis[2 * i];
            const double v_im = w_i * (double)job->vis[2 * i + 1];
            const size_t kstart = (size_t)p->plane * job->plane_stride;
            const int s = p->support;
            for (j = j0; j <= j1; ++j)
            {
                const size_t row = (size_t)(p->gv + j) * (size_t)G +
                        (size_t)p->gu;
                const size_t krow = kstart +
                        (size_t)abs(p->ov + j * os) * job->conv_size_half;
                for (k = -s; k <= s; ++k)
                {
                    const size_t t = (krow + abs(p->ou + k * os)) << 1;
                    const size_t c = (row + k) << 1;
                    const double c_re = job->conv_func[t];
                    const double c_im = (double)job->conv_func[t + 1] * conj;
                    job->grid64[c]     += (v_re * c_re - v_im * c_im);
                    job->grid64[c + 1] += (v_im * c_re + v_re * c_im);
                }
            }
        }
        else
        {
            const float conj = p->conj_neg ? -1.0f : 1.0f;
            const float w_i = job->weight[i];
            const float v_re = w_i * job->vis[2 * i];
            const float v_im = w_i * job->vis[2 * i + 1];
            const size_t kstart = (size_t)p->plane * job->plane_stride;
            const int s = p->support;
            for (j = j0; j <= j1; ++j)
            {
                const size_t row = (size_t)(p->gv + j) * (size_t)G +
                        (size_t)p->gu;
                const size_t krow = kstart +
                        (size_t)abs(p->ov + j * os) * job->conv_size_half;
                for (k = -s; k <= s; ++k)
                {
                    const size_t t = (krow + abs(p->ou + k * os)) << 1;
                    const size_t c = (row + k) << 1;
                    const float c_re = job->conv_func[t];
                    const float c_im = job->conv_func[t + 1] * conj;
                    job->grid[c]     += (v_re * c_re - v_im * c_im);
                    job->grid[c + 1] += (v_im * c_re + v_re * c_im);
                }
            }
        }
    }
}

static void* mt_worker(void* arg)
{
    mt_job_t* job = (mt_job_t*)arg;
    for (;;)
    {
        const int item = __atomic_fetch_add(&job->next, 1, __ATOMIC_RELAXED);
        if (job->phase == 0)
        {
            const size_t i0 = (size_t)item * job->chunk;
            size_t i1;
            if (i0 >= job->num_points) break;
            i1 = i0 + job->chunk;
            if (i1 > job->num_points) i1 = job->num_points;
            mt_place_chunk(job, i0, i1);
        }
        else
        {
            if (item >= job->num_bands) break;
            mt_grid_band(job, item);
        }
    }
    return NULL;
}

static void mt_run(mt_job_t* job, int num_threads)
{
    int t;
    pthread_t* th = (pthread_t*)calloc((size_t)num_threads, sizeof(pthread_t));
    job->next = 0;
    for (t = 1; t < num_threads; ++t)
        pthread_create(&th[t], NULL, mt_worker, job);
    mt_worker(job);
    for (t = 1; t < num_threads; ++t)
        pthread_join(th[t], NULL);
    free(th);
}

static int mt_grid(int num_threads, size_t num_w_planes,
        const int* support, int oversample, int conv_size_half,
        const float* conv_func, size_t num_points, const float* uu,
        const float* vv, const float* ww, const float* vis,
        const float* weight, float cell_size_rad, float w_scale,
        int grid_size, size_t* num_skipped, double* norm, float* grid,
        double* grid64, int place64)
{
    size_t i, n_skip = 0;
    mt_job_t job;
    if (num_threads < 1) num_threads = 1;
    memset(&job, 0, sizeof(job));
    job.place = (oracle_place_t*)malloc(
            (num_points ? num_points : 1) * sizeof(oracle_place_t));
    job.tap_sum = (double*)malloc((num_points ? num_points : 1) *
            sizeof(double));
    if (!job.place || !job.tap_sum)
    {
        free((void*)job.place); free(job.tap_sum);
        return -1;
    }
    job.conv_func = conv_func; job.vis = vis; job.weight = weight;
    job.grid = grid; job.grid64 = grid64; job.num_points = num_points;
    job.place64 = place64;
    job.plane_stride = (size_t)(conv_size_half * conv_size_half);
    job.oversample = oversample; job.conv_size_half = conv_size_half;
    job.grid_size = grid_size;
    job.uu = uu; job.vv = vv; job.ww = ww; job.support = support;
    job.num_w_planes = num_w_planes;
    job.cell_size_rad = cell_size_rad; job.w_scale = w_scale;
    job.chunk = 4096;
    /* Enough bands that the dense centre spreads over many threads. */
    job.num_bands = num_threads * 8;
    if (job.num_bands > grid_size) job.num_bands = grid_size;
    if (job.num_bands < 1) job.num_bands = 1;

    job.phase = 0;
    mt_run(&job, num_threads);
    job.phase = 1;
    mt_run(&job, num_threads);

    for (i = 0; i < num_points; ++i)
    {
        if (job.place[i].skipped) { n_skip++; continue; }
        *norm += job.tap_sum[i] * weight[i];
    }
    *num_skipped = n_skip;
    free((void*)job.place);
    free(job.tap_sum);
    return 0;
}

/* Same arguments and results as oracle_grid_wproj_f, run on num_threads
 * host threads.  Returns 0, or -1 when scratch memory cannot be had. */
ORACLE_API int oracle_grid_wproj_f_mt(int num_threads, size_t num_w_planes,
        const int* support, int oversample, int conv_size_half,
        const float* conv_func, size_t num_points, const float* uu,
        const float* vv, const float* ww, const float* vis,
        const float* weight, float cell_size_rad, float w_scale,
        int grid_size, size_t* num_skipped, double* norm, float* grid)
{
    return mt_grid(num_threads, num_w_planes, support, oversample,
            conv_size_half, conv_func, num_points, uu, vv, ww, vis, weight,
            cell_size_rad, w_scale, grid_size, num_skipped, norm, grid, NULL,
            0);
}

/* oracle_grid_wproj_f_fp64acc on num_threads host threads: every cell
 * receives its FP64 contributions in input order, so the grid and the norm
 * are bit-identical to the serial function's.  Returns 0, or -1 when scratch
 * memory cannot be had. */
ORACLE_API int oracle_grid_wproj_f_fp64acc_mt(int num_threads,
        size_t num_w_planes, const int* support, int oversample,
        int conv_size_half, const float* conv_func, size_t num_points,
        const float* uu, const float* vv, const float* ww, const float* vis,
        const float* weight, float cell_size_rad, float w_scale,
        int grid_size, size_t* num_skipped, double* norm, double* grid)
{
    return mt_grid(num_threads, num_w_planes, support, oversample,
            conv_size_half, conv_func, num_points, uu, vv, ww, vis, weight,
            cell_size_rad, w_scale, grid_size, num_skipped, norm, NULL, grid,
            0);
}

/* oskar_grid_wproj_d (oskar_grid_wproj.c:37-123) on FP32 inputs promoted
 * to FP64 -- coordinates, visibilities, weights, kernel cube, cell size and
 * w scale -- run on num_threads host threads: FP64 placement, FP64 sums in
 * input order per cell, so grid and norm are bit-identical to the serial
 * oracle_grid_wproj_d (and the reference's _d) on the promoted arrays.  This
 * is the reference's own FP64 answer for an FP32 workload; where its FP64
 * placement puts a visibility in another cell, offset or plane than the
 * FP32 rules do, it differs from oracle_grid_wproj_f_fp64acc_mt by that
 * visibility's contribution.  Returns 0, or -1 when scratch memory cannot
 * be had. */
ORACLE_API int oracle_grid_wproj_d_promoted_mt(int num_threads,
        size_t num_w_planes, const int* support, int oversample,
        int conv_size_half, const float* conv_func, size_t num_points,
        const float* uu, const float* vv, const float* ww, const float* vis,
        const float* weight, float cell_size_rad, float w_scale,
        int grid_size, size_t* num_skipped, double* norm, double* grid)
{
    return mt_grid(num_threads, num_w_planes, support, oversample,
            conv_size_half, conv_func, num_points, uu, vv, ww, vis, weight,
            cell_size_rad, w_scale, grid_size, num_skipped, norm, NULL, grid,
            1);
}

/* ------------------------------------------------------------------------ */
/* Uniform-weighting density (the step before gridding)                     */
/* ------------------------------------------------------------------------ */

/* Restatement of oskar_grid_weights_write_f, utils/oskar_grid_weights.c:
 * 106-138: nearest-cell accumulation of the weights. */
ORACLE_API void oracle_grid_weights_write_f(size_t num_points,
        const float* uu, const float* vv, const float* weight,
        float cell_size_rad, int grid_size, size_t* num_skipped, float* grid)
{
    size_t i, n_skip = 0;
    const int centre = grid_size / 2;
    const float scale = grid_size * cell_size_rad;
    for (i = 0; i < num_points; ++i)
    {
        const int gu = (int)roundf(-uu[i] * scale) + centre;
        const int gv = (int)roundf(vv[i] * scale) + centre;
        if (gu >= grid_size || gu < 0 || gv >= grid_size || gv < 0)
        {
            n_skip++;
            continue;
        }
        grid[(size_t)gv * (size_t)grid_size + (size_t)gu] += weight[i];
    }
    *num_skipped = n_skip;
}

/* Restatement of oskar_grid_weights_read_f, utils/oskar_grid_weights.c:
 * 140-172: weight_out = weight_in / density, or 0 where the density is 0.
 * Skipped points leave weight_out untouched, as the reference does. */
ORACLE_API void oracle_grid_weights_read_f(size_t num_points,
        const float* uu, const float* vv, const float* weight_in,
        float* weight_out, float cell_size_rad, int grid_size,
        size_t* num_skipped, const float* grid)
{
    size_t i, n_skip = 0;
    const int centre = grid_size / 2;
    const float scale = grid_size * cell_size_rad;
    for (i = 0; i < num_points; ++i)
    {
        const int gu = (int)roundf(-uu[i] * scale) + centre;
        const int gv = (int)roundf(vv[i] * scale) + centre;
        float d;
        if (gu >= grid_size || gu < 0 || gv >= grid_size || gv < 0)
        {
            n_skip++;
            continue;
        }
        d = grid[(size_t)gv * (size_t)grid_size + (size_t)gu];
        /* The reference compares and divides with a double 0.0 literal:
         * weight_in / d is FP32, the 0.0 branch converts to FP32. */
        weight_out[i] = (d != 0.0) ? weight_in[i] / d : 0.0;
    }
    *num_skipped = n_skip;
}

/* FP64 versions, utils/oskar_grid_weights.c:38-104. */
ORACLE_API void oracle_grid_weights_write_d(size_t num_points,
        const double* uu, const double* vv, const double* weight,
        double cell_size_rad, int grid_size, size_t* num_skipped,
        double* grid)
{
    size_t i, n_skip = 0;
    const int centre = grid_size / 2;
    const double scale = grid_size * cell_size_rad;
    for (i = 0; i < num_points; ++i)
    {
        const int gu = (int)round(-uu[i] * scale) + centre;
        const int gv = (int)round(vv[i] * scale) + centre;
        if (gu >= grid_size || gu < 0 || gv >= grid_size || gv < 0)
        {
            n_skip++;
            continue;
        }
        grid[(size_t)gv * (size_t)grid_size + (size_t)gu] += weight[i];
    }
    *num_skipped = n_skip;
}

ORACLE_API void oracle_grid_weights_read_d(size_t num_points,
        const double* uu, const double* vv, const double* weight_in,
        double* weight_out, double cell_size_rad, int grid_size,
        size_t* num_skipped, const double* grid)
{
    size_t i, n_skip = 0;
    const int centre = grid_size / 2;
    const double scale = grid_size * cell_size_rad;
    for (i = 0; i < num_points; ++i)
    {
        const int gu = (int)round(-uu[i] * scale) + centre;
        const int gv = (int)round(vv[i] * scale) + centre;
        double d;
        if (gu >= grid_size || gu < 0 || gv >= grid_size || gv < 0)
        {
            n_skip++;
            continue;
        }
        d = grid[(size_t)gv * (size_t)grid_size + (size_t)gu];
        weight_out[i] = (d != 0.0) ? weight_in[i] / d : 0.0;
    }
    *num_skipped = n_skip;
}
