/*
 * gpugrid.h -- C ABI of the GB300 W-projection gridder (libgpugrid.so).
 *
 * The library is a drop-in for the reference's serial gridding functions
 * (oskar_grid_wproj.h:69-86 and :114-131 of the reference project) plus the
 * entry points a GPU caller needs: status codes, device-pointer variants on
 * a caller's CUDA stream, reusable kernel-stack handles, a batched
 * multi-channel path, the adjoint (degridding) map and the uniform-weighting
 * density step.  Every signature uses plain pointers, sizes and scalars;
 * streams are passed as `void*` (a cudaStream_t, NULL for the legacy default
 * stream) so this header needs no CUDA include.
 *
 * Threading: calls may come from several host threads; work for one device
 * is serialised by a per-device lock.  Results are deterministic: the same
 * inputs give bit-identical grids, norms and counts on every call.
 */
#ifndef GPUGRID_H_
#define GPUGRID_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define GG_API __attribute__((visibility("default")))
#else
#define GG_API
#endif

/* Status codes returned by every gg_* entry point that returns int. */
enum
{
    GG_OK = 0,
    GG_ERR_INVALID_ARG = 1,   /* a size, pointer or parameter is invalid */
    GG_ERR_CUDA = 2,          /* a CUDA runtime call failed */
    GG_ERR_NO_MEMORY = 3,     /* a device or host allocation failed */
    GG_ERR_UNSUPPORTED = 4,   /* valid input outside this build's limits */
    GG_ERR_CAPACITY = 5       /* a reserved workspace was too small */
};

/* ---------------------------------------------------------------------- */
/* Drop-in replacements                                                   */
/* ---------------------------------------------------------------------- */

/* Same signature and semantics as oskar_grid_wproj_d (reference
 * oskar_grid_wproj.h:69-86, oskar_grid_wproj.c:37-123).  Host pointers;
 * synchronous; *num_skipped is set, *norm and grid are accumulated.  FP64
 * placement and FP64 accumulation on the GPU.  On failure the outputs are
 * left untouched and gg_last_error() describes the failure. */
GG_API void oskar_grid_wproj_d(const size_t num_w_planes, const int* support,
        const int oversample, const int conv_size_half,
        const double* conv_func, const size_t num_points, const double* uu,
        const double* vv, const double* ww, const double* vis,
        const double* weight, const double cell_size_rad,
        const double w_scale, const int grid_size, size_t* num_skipped,
        double* norm, double* grid);

/* Same signature and semantics as oskar_grid_wproj_f (reference
 * oskar_grid_wproj.h:114-131, oskar_grid_wproj.c:126-212).  Placement,
 * plane choice and num_skipped are bit-exact with the reference's FP32 rules;
 * the grid is accumulated in compensated FP32; norm is FP64. */
GG_API void oskar_grid_wproj_f(const size_t num_w_planes, const int* support,
        const int oversample, const int conv_size_half,
        const float* conv_func, const size_t num_points, const float* uu,
        const float* vv, const float* ww, const float* vis,
        const float* weight, const float cell_size_rad, const float w_scale,
        const int grid_size, size_t* num_skipped, double* norm, float* grid);

/* Status-returning forms of the two drop-ins (same arguments). */
GG_API int gg_grid_wproj_d(size_t num_w_planes, const int* support,
        int oversample, int conv_size_half, const double* conv_func,
        size_t num_points, const double* uu, const double* vv,
        const double* ww, const double* vis, const double* weight,
        double cell_size_rad, double w_scale, int grid_size,
        size_t* num_skipped, double* norm, double* grid);
GG_API int gg_grid_wproj_f(size_t num_w_planes, const int* support,
        int oversample, int conv_size_half, const float* conv_func,
        size_t num_points, const float* uu, const float* vv,
        const float* ww, const float* vis, const float* weight,
        float cell_size_rad, float w_scale, int grid_size,
        size_t* num_skipped, double* norm, float* grid);

/* Message for the last failure on the calling host thread ("" if none). */
GG_API const char* gg_last_error(void);

/* Library version string. */
GG_API const char* gg_version(void);

/* ---------------------------------------------------------------------- */
/* Kernel stacks (re-laid, device-resident W-kernel cubes)                */
/* ---------------------------------------------------------------------- */

/* A kernel stack is the reference's (support, oversample, conv_size_half,
 * conv_func) tuple (oskar_grid_wproj.h:114-119) uploaded once and re-laid on
 * the device for the gridding kernels, together with the per-plane,
 * per-offset FP64 tap sums used for the norm.  The handle owns its device
 * memory; the caller may change or free conv_func after creation.  It is
 * tied to the device current at creation. */
typedef struct gg_kernels gg_kernels;

/* conv_func_on_device = 0: conv_func is host memory; 1: device memory.
 * support is always host memory.  stream: cudaStream_t or NULL. */
GG_API int gg_kernels_create_f(gg_kernels** out, size_t num_w_planes,
        const int* support, int oversample, int conv_size_half,
        const float* conv_func, int conv_func_on_device, void* stream);
GG_API int gg_kernels_create_d(gg_kernels** out, size_t num_w_planes,
        const int* support, int oversample, int conv_size_half,
        const double* conv_func, int conv_func_on_device, void* stream);
/* A kernel stack generated on the device, so that no cube crosses the host
 * link: plane p of the cube is the taper x chirp kernel the synthetic
 * workloads of this project use,
 *   k(iv, iu) = exp(-2 (r2 / os^2) / s_p^2) * exp(i pi w_p r2 / csh^2),
 *   r2 = iv^2 + iu^2 (oversampled pixels), s_p = max(support[p], 1),
 * divided by the complex sum of the taps a visibility at zero offset uses
 * (k[|j| os][|l| os], |j|, |l| <= s_p, inside the cube), computed in FP64
 * and rounded once.  w_planes: host array of the P chirp parameters w_p.
 * d_conv_func_out (device, [P][csh][csh] complex) receives the cube when
 * not NULL.  The reference reads its kernels from FITS files instead
 * (utils/read_kernel.c:36-118). */
GG_API int gg_kernels_generate_f(gg_kernels** out, size_t num_w_planes,
        const int* support, int oversample, int conv_size_half,
        const double* w_planes, float* d_conv_func_out, void* stream);
GG_API int gg_kernels_generate_d(gg_kernels** out, size_t num_w_planes,
        const int* support, int oversample, int conv_size_half,
        const double* w_planes, double* d_conv_func_out, void* stream);
GG_API int gg_kernels_destroy(gg_kernels* k);

/* ---------------------------------------------------------------------- */
/* Device-pointer gridding                                                */
/* ---------------------------------------------------------------------- */

/* A plan owns the device workspace (placement arrays, sort buffers, work
 * items, partial tiles) and grows it on demand.  One plan serves one call
 * at a time; use one plan per concurrent stream. */
typedef struct gg_plan gg_plan;

GG_API int gg_plan_create(gg_plan** out);
GG_API int gg_plan_destroy(gg_plan* plan);

/* Statistics of the last call made with a plan (valid after the stream
 * has been synchronised). */
typedef struct
{
    unsigned long long num_points;
    unsigned long long num_skipped;
    unsigned long long num_records;     /* (visibility, tile) pairs */
    unsigned long long num_macs;        /* complex multiply-adds performed */
    unsigned long long num_launches;    /* kernels this library launched */
    int tile_u, tile_v;                 /* tile shape used */
    int slice_staging;                  /* 1 if slices were staged */
    int num_ctas;                       /* persistent gridding CTAs */
    unsigned long long chunk_records;   /* records per work item (max) */
    int num_plane_groups;               /* gridding passes (plane groups) */
} gg_stats;

GG_API int gg_plan_last_stats(const gg_plan* plan, gg_stats* stats);

/* Tile shape of the gridding kernel for calls made with this plan.  Every
 * tile holds 2048 cells: tile_u = 32 (32 x 64 cells), 16 (16 x 128) or 8
 * (8 x 256); 0 (the default) lets each call choose from its mean footprint
 * (narrow tiles for small supports).  The result of a call depends only on
 * its inputs and this setting. */
GG_API int gg_plan_set_tile_shape(gg_plan* plan, int tile_u);

/* Staging of kernel slices in shared memory by the gridding kernel (bulk
 * asynchronous copies of a (plane, offset) slice shared by many records of
 * a tile): -1 (default) decides per call from the mean footprint, 0 off,
 * 1 on.  Results are bit-identical either way: only where the taps are
 * read from changes, not the arithmetic or its order. */
GG_API int gg_plan_set_slice_staging(gg_plan* plan, int mode);

/* Launch and decomposition parameters of a plan's gridding calls, as set
 * by an autotuner (or by hand).  Every setting changes speed only:
 * placement, norm and num_skipped are the same under all of them.  The
 * settings that change how a cell's contributions are grouped or ordered
 * (tile_u, items_per_cta, sort_detail, ctas_per_sm -- through the number of
 * work items --, plane_group_mb, tile_phases) change the grid by FP32
 * rounding; slice_staging leaves it bit-identical.
 *   tile_u         32, 16 or 8 (cells across a tile); 0 = chosen per call
 *   slice_staging  -1 chosen per call, 0 off, 1 on (bit-identical results)
 *   items_per_cta  work items per persistent CTA in each gridding pass
 *                  that the split of heavy tiles aims for, 1..64 (default
 *                  4): more items balance the load better but write more
 *                  partial tiles
 *   sort_detail    order of a tile's records: 2 (default) by w-plane then
 *                  kernel-offset class, 1 by w-plane, 0 visibility order
 *   ctas_per_sm    resident gridding CTAs per SM, 0 (default) = as many as
 *                  fit, else min(that, what fits), 1..32
 *   plane_group_mb kernel bytes per gridding pass: the w-planes are cut
 *                  into as few groups of consecutive planes as keep each
 *                  group's re-laid kernels within this many MiB (about
 *                  equal in size) and each group is gridded in its own
 *                  pass, so that a pass's kernels stay in L2; 0 (default) =
 *                  half the device's L2 cache, 0..1048576
 *   tile_order     order in which the persistent CTAs take the tiles: 0
 *                  (default) by distance from the grid centre (baseline
 *                  length, so w and the kernels read stay alike among the
 *                  tiles gridded at one time), 1 row by row (the tiles in
 *                  flight share grid rows: fewer pages touched at once when
 *                  the grid is the caller's host memory, used in place)
 *   lane_groups    record streams per consumer warp of the 32-wide tiles
 *                  (taps read from the slab stack): 1 -- the whole warp
 *                  takes every record that meets its 8 rows; 2 -- each
 *                  half-warp takes the records that meet its own 16
 *                  columns, so two narrow footprints are gridded side by
 *                  side; 0 (default) = 1
 *   tile_phases    1, 2, 4 or 8 tile grids offset by tile_u / tile_phases
 *                  columns from one another; each visibility is gridded on
 *                  the one whose tiles cut its footprint into the fewest
 *                  columns (fewer lanes outside footprints, fewer records),
 *                  all in one pass per plane group (the tiles of later
 *                  grids add partial tiles after it); 0 (default): four
 *                  when the call's mean footprint is narrower than the
 *                  tile, else one
 * gg_plan_set_tile_shape and gg_plan_set_slice_staging set the first two
 * fields alone. */
typedef struct
{
    int tile_u;
    int slice_staging;
    int items_per_cta;
    int sort_detail;
    int ctas_per_sm;
    int plane_group_mb;
    int tile_order;
    int lane_groups;
    int tile_phases;
} gg_tuning;

GG_API int gg_plan_set_tuning(gg_plan* plan, const gg_tuning* tuning);
GG_API int gg_plan_get_tuning(const gg_plan* plan, gg_tuning* tuning);

/* Tuning of the host-pointer entry points (oskar_grid_wproj_f/_d and
 * gg_grid_wproj_f/_d) on the current device: they keep one workspace plan
 * per device, and this sets its gg_tuning (NULL restores the defaults).
 * An integrator sets it once, e.g. from an autotuned plan for the
 * production grid; results are the same under every tuning. */
GG_API int gg_host_set_tuning(const gg_tuning* tuning);
GG_API int gg_host_get_tuning(gg_tuning* tuning);

/* How the host-pointer gridding and degridding calls on the current device
 * reach the caller's grid and kernel cube (degridding only reads the
 * grid: in place, each work item loads its tile once).
 *   GG_GRID_ACCESS_COPY:     both are copied to the device (the cube's read
 *                            squares by 3-D copies); the grid is gridded
 *                            there and the rows' spans that hold records
 *                            are copied back.
 *   GG_GRID_ACCESS_PINNED:   page-locked arrays that the device can address
 *                            (cudaHostAlloc / cudaMallocHost,
 *                            cudaHostRegister with mapping) are used in
 *                            place: the gridding kernels read each tile that
 *                            holds records once and write it once over the
 *                            host link during the gridding passes, and a
 *                            kernel gathers the cube's read squares.  Other
 *                            arrays are copied.
 *   GG_GRID_ACCESS_PAGEABLE: (default) as PINNED, and pageable (malloc)
 *                            arrays too where the device reads pageable
 *                            memory through the host's page tables
 *                            (cudaDevAttrPageableMemoryAccess and
 *                            ...UsesHostPageTables, e.g. Grace hosts) and
 *                            every page of the array is resident (mincore):
 *                            a page first touched by the device is faulted
 *                            in at some 25 us, so a freshly allocated zero
 *                            grid is copied.
 * An array must be aligned to its complex element (8 bytes for _f, 16 for
 * _d) to be used in place.  The grid is written in place, so it must be
 * writable memory (as it must for any mode: it is accumulated): never a
 * read-only mapping or a cudaHostRegisterReadOnly registration, which the
 * device could not write; use GG_GRID_ACCESS_COPY for such arrays.  The grid in place is bit-identical to the
 * device-pointer call's; copied, it is too on grids under 128 MiB (above,
 * the copy's split passes change the rounding only). */
enum {
    GG_GRID_ACCESS_COPY = 0,
    GG_GRID_ACCESS_PINNED = 1,
    GG_GRID_ACCESS_PAGEABLE = 2
};
GG_API int gg_host_set_grid_access(int mode);
GG_API int gg_host_get_grid_access(int* mode);

/* Phase timing of the host-pointer gridding calls on the current device.
 * With profiling enabled, gg_host_phase_ms fills ms[0..n-1] (n <= 9) for
 * the last such call that gridded at least one visibility:
 *   0 staging: the call's start to placement (kernel stack re-layout, the
 *     inputs' upload)
 *   1-4 the phases 0-3 of gg_plan_phase_ms (placement, binning, work
 *     decomposition, tile-gridding passes)
 *   5 the rest: the end of the passes to the end of the call (grid copy
 *     back, scalars).
 * and, measured on the host clock:
 *   6 the call's entry to its first queued device work (checks, host-array
 *     classification, buffers)
 *   7 the call's entry to the return of its final synchronisation
 *   8 the whole call, entry to return.
 * Off by default (no events recorded). */
GG_API int gg_host_set_profiling(int enable);
GG_API int gg_host_phase_ms(float* ms, int n);

/* Bytes the last host-pointer gridding call on the current device moved
 * host -> device (kernel cube and plane tables, the call's arrays, the
 * grid or, in place, the cells of the tiles that hold records, norm) and
 * device -> host (the grid rows' spans that hold records or, in place, the
 * same tiles' cells, norm, skip count and a few status words); 0, 0 before
 * the first call. */
GG_API int gg_host_last_transfer(unsigned long long* h2d_bytes,
                                 unsigned long long* d2h_bytes);

/* Host-clock marks (ms from the call's entry) of the last host-pointer
 * gridding call on the current device, profiled or not: ms[0] its first
 * queued device work, ms[1] the return of its final synchronisation, ms[2]
 * its return (n <= 3 are filled; zeros before the first call). */
GG_API int gg_host_last_call_ms(double* ms, int n);

/* Phase timing.  With profiling enabled, every gridding call made with the
 * plan records CUDA events on its stream around five phases:
 *   0 placement (placement, skip/norm reduction, record offsets)
 *   1 binning (record emission and radix sort)
 *   2 work decomposition (tile ranges and work items)
 *   3 the tile-gridding passes (one per plane group, each with the
 *     reduction of its split tiles' partials)
 *   4 reserved (0; the reductions are timed within phase 3)
 * gg_plan_phase_ms fills ms[0..n-1] for the last call; the call's stream
 * must have been synchronised.  Off by default (no events recorded). */
GG_API int gg_plan_set_profiling(gg_plan* plan, int enable);
GG_API int gg_plan_phase_ms(const gg_plan* plan, float* ms, int n);

/* Measured FP32 fused-multiply-add throughput of the current device, in
 * TFLOP/s (2 FLOP per FMA): the roofline denominator of the FP32 gridding
 * kernel.  Runs for a few tens of milliseconds. */
GG_API int gg_measure_fp32_fma_tflops(double* tflops);

/* Grid num_points visibilities held in device memory onto a device grid.
 * Semantics are those of oskar_grid_wproj_f with device pointers:
 * *d_num_skipped (device, 64-bit) is set, *d_norm (device) and d_grid
 * (device, complex64 grid_size^2, row-major with v as the row) are
 * accumulated.  Runs on `stream`; the call returns once the work is queued
 * (it synchronises the stream once, to size the sort buffers). */
GG_API int gg_grid_wproj_f_device(gg_plan* plan, const gg_kernels* kernels,
        size_t num_points, const float* d_uu, const float* d_vv,
        const float* d_ww, const float* d_vis, const float* d_weight,
        float cell_size_rad, float w_scale, int grid_size,
        unsigned long long* d_num_skipped, double* d_norm, float* d_grid,
        void* stream);
GG_API int gg_grid_wproj_d_device(gg_plan* plan, const gg_kernels* kernels,
        size_t num_points, const double* d_uu, const double* d_vv,
        const double* d_ww, const double* d_vis, const double* d_weight,
        double cell_size_rad, double w_scale, int grid_size,
        unsigned long long* d_num_skipped, double* d_norm, double* d_grid,
        void* stream);

/* Batched gridding: num_grids independent grids (frequency channels or
 * snapshots, each with its own number of visibilities) in one call -- one
 * placement pass, one sort and one persistent tile-gridding launch over all
 * of them.  Grid g takes visibilities [offsets[g], offsets[g+1]) of the
 * concatenated device arrays d_uu ... d_weight (offsets: host, num_grids+1
 * entries, offsets[0] = 0) and accumulates into d_grids + g * grid_size^2 *
 * 2; d_norm[g] is accumulated and d_num_skipped[g] set (device arrays of
 * num_grids).  The kernel stack, cell size and w_scale are shared.  Each
 * grid's result equals that of gg_grid_wproj_f_device on its own
 * visibilities (same placement, norm and num_skipped; grid within FP32
 * rounding).  The reference grids one channel per call (its main.cpp
 * loops over visibility blocks and calls oskar_grid_wproj_f for each). */
GG_API int gg_grid_wproj_f_batched_device(gg_plan* plan,
        const gg_kernels* kernels, int num_grids,
        const unsigned long long* offsets, const float* d_uu,
        const float* d_vv, const float* d_ww, const float* d_vis,
        const float* d_weight, float cell_size_rad, float w_scale,
        int grid_size, unsigned long long* d_num_skipped, double* d_norm,
        float* d_grids, void* stream);
GG_API int gg_grid_wproj_d_batched_device(gg_plan* plan,
        const gg_kernels* kernels, int num_grids,
        const unsigned long long* offsets, const double* d_uu,
        const double* d_vv, const double* d_ww, const double* d_vis,
        const double* d_weight, double cell_size_rad, double w_scale,
        int grid_size, unsigned long long* d_num_skipped, double* d_norm,
        double* d_grids, void* stream);

/* Replay of a plan's last batched call on new amplitudes and weights.  The
 * plan keeps the geometry of its last successful batched call (placement,
 * sorted records, work items, tile shape); a replay grids d_vis and
 * d_weight -- laid out like that call's inputs, same number of
 * visibilities -- with it, for imaging loops whose (u, v, w) coordinates
 * stay fixed while the amplitudes change between major cycles.  Outputs as
 * in the batched call (grids and d_norm accumulated, d_num_skipped set);
 * with the original amplitudes and weights the results are bit-identical
 * to the batched call's.  A replay only enqueues kernel launches and a
 * memset on the stream -- no allocation, no host synchronisation -- so it
 * may be captured in a CUDA graph.  Any other gridding call on the plan
 * discards the kept geometry (GG_ERR_INVALID_ARG on the next replay).  The
 * kernels argument must be the batched call's.  A failure inside the
 * gridding kernel (a bounded wait that ran out) is reported by the next
 * gg_plan_check or the next non-replay call. */
GG_API int gg_grid_wproj_f_batched_replay(gg_plan* plan,
        const gg_kernels* kernels, const float* d_vis, const float* d_weight,
        unsigned long long* d_num_skipped, double* d_norm, float* d_grids,
        void* stream);
GG_API int gg_grid_wproj_d_batched_replay(gg_plan* plan,
        const gg_kernels* kernels, const double* d_vis,
        const double* d_weight, unsigned long long* d_num_skipped,
        double* d_norm, double* d_grids, void* stream);

/* Largest number of visibilities one sub-batch of a batched call takes.
 * A batched call is cut, between grids, into sub-batches of consecutive
 * grids whenever its (visibility, tile) records might not fit the 32-bit
 * record indices of one sort -- more than (2^32 - 16) / r visibilities,
 * r = (2 s_max / tile_u + 2) * (2 s_max / tile_v + 2), taken over the tile
 * shapes the plan may choose -- or exceed this limit (0, the default: no
 * further limit).  Each sub-batch is gridded by a sub-plan that keeps its
 * geometry, so replays cover every grid; the sort's transient buffers are
 * shared, so smaller sub-batches need less workspace.  A single grid above
 * the limit is refused with GG_ERR_UNSUPPORTED. */
GG_API int gg_plan_set_batch_limit(gg_plan* plan,
                                   unsigned long long max_points);

/* Synchronises the stream and returns GG_ERR_CUDA if a gridding kernel of
 * this plan flagged a failure (a bounded wait that ran out). */
GG_API int gg_plan_check(gg_plan* plan, void* stream);

/* Diagnostic of that failure path, safe to run: a kernel waits, bounded by
 * `iterations` probes (1..1048576, each failed probe sleeping ~64 ns), on
 * an mbarrier that nothing arrives at -- the kind of wait the gridding
 * kernels bound -- so the wait runs out, the kernel sets the plan's error
 * flag and returns.  Returns GG_ERR_CUDA (with its message) as the plan
 * then does from every call; the device and other plans stay usable. */
GG_API int gg_plan_probe_bounded_wait(gg_plan* plan, unsigned iterations,
                                      void* stream);

/* Allocation-free form of gg_grid_wproj_f_device, for callers that cannot
 * allocate device memory while they grid (a real-time loop that must not
 * stall on cudaMalloc, or code running under another framework's memory
 * pool).  This entry point has no counterpart in the reference.  All scratch
 * comes from one 32 MiB device array inside the library, held by every GPU
 * that loads it until the process exits; nothing is allocated or freed by
 * the call.  The kernel-stack handle is made beforehand (that step
 * allocates).  Limits: num_points <= 131072, grid_size <= 8192, and at most
 * 1048576 (visibility, tile) records; beyond them the call returns
 * GG_ERR_CAPACITY and leaves the grid, *d_norm and *d_num_skipped untouched
 * (so a caller may split the call and retry).  All calls on a device share
 * the array, so calls that overlap on the GPU race and must be serialised by
 * the caller.  The first call on each device looks up the array's device
 * address; make it with that device current and before any stream capture.
 * If a call's gridding kernel runs out of its bounded wait (see
 * gg_plan_check), that call has already returned GG_OK: the failure is
 * reported by the next no-alloc call on the same device, which returns
 * GG_ERR_CUDA with its outputs untouched and clears the flag -- the
 * incomplete grid is the earlier call's.  Same semantics and results as
 * gg_grid_wproj_f_device otherwise (grid and *d_norm accumulated,
 * *d_num_skipped set; one stream synchronisation per call). */
GG_API int gg_grid_wproj_f_device_noalloc(const gg_kernels* kernels,
        size_t num_points, const float* d_uu, const float* d_vv,
        const float* d_ww, const float* d_vis, const float* d_weight,
        float cell_size_rad, float w_scale, int grid_size,
        unsigned long long* d_num_skipped, double* d_norm, float* d_grid,
        void* stream);

/* Diagnostic of the no-alloc failure report, safe to run: the bounded wait
 * of gg_plan_probe_bounded_wait, run out on purpose against the no-alloc
 * array's error flag on the current device, so that the next
 * gg_grid_wproj_f_device_noalloc call on it reports GG_ERR_CUDA.  No
 * counterpart in the reference.  iterations in 1..1048576. */
GG_API int gg_noalloc_probe_bounded_wait(unsigned iterations, void* stream);

/* Placement only (diagnostic): writes, per visibility, six int32 --
 * cell u, cell v, off_u, off_v, w-plane (after the clamp to the last plane)
 * and flags (bit 0 skipped, bit 1 kernel conjugated because ww > 0) --
 * exactly as the gridding entry points compute them.  This is the
 * per-visibility state of reference oskar_grid_wproj.c:155-187 (FP32 rules)
 * and :66-98 (FP64 rules).  d_out: device int32[6 * num_points]. */
GG_API int gg_place_wproj_f_device(const gg_kernels* kernels,
        size_t num_points, const float* d_uu, const float* d_vv,
        const float* d_ww, float cell_size_rad, float w_scale, int grid_size,
        int* d_out, void* stream);
GG_API int gg_place_wproj_d_device(const gg_kernels* kernels,
        size_t num_points, const double* d_uu, const double* d_vv,
        const double* d_ww, double cell_size_rad, double w_scale,
        int grid_size, int* d_out, void* stream);

/* ---------------------------------------------------------------------- */
/* Adjoint (degridding)                                                   */
/* ---------------------------------------------------------------------- */

/* The exact adjoint of the map v -> grid that oskar_grid_wproj_f applies
 * to the weighted visibilities v_i = weight_i * vis_i (reference
 * oskar_grid_wproj.c:190-209 defines the forward map; the reference has no
 * degridder):  d_out_vis[i] = sum over the footprint of
 * conj(c~_i(cell)) * d_grid(cell), with c~ the tap whose imaginary part is
 * negated for ww > 0, and the same placement rules as the forward call.
 * Skipped visibilities get 0.  Device pointers, complex interleaved. */
GG_API int gg_degrid_wproj_f_device(gg_plan* plan, const gg_kernels* kernels,
        size_t num_points, const float* d_uu, const float* d_vv,
        const float* d_ww, float cell_size_rad, float w_scale, int grid_size,
        const float* d_grid, float* d_out_vis, void* stream);
GG_API int gg_degrid_wproj_d_device(gg_plan* plan, const gg_kernels* kernels,
        size_t num_points, const double* d_uu, const double* d_vv,
        const double* d_ww, double cell_size_rad, double w_scale,
        int grid_size, const double* d_grid, double* d_out_vis, void* stream);

/* Host-pointer degridding, the sibling of oskar_grid_wproj_f/_d (the
 * reference has no degridder): the same kernel stack, coordinates and
 * placement rules; vis (complex interleaved, num_points entries) is
 * overwritten with the adjoint map above applied to grid.  Synchronous. */
GG_API int gg_degrid_wproj_f(size_t num_w_planes, const int* support,
        int oversample, int conv_size_half, const float* conv_func,
        size_t num_points, const float* uu, const float* vv, const float* ww,
        float cell_size_rad, float w_scale, int grid_size, const float* grid,
        float* vis);
GG_API int gg_degrid_wproj_d(size_t num_w_planes, const int* support,
        int oversample, int conv_size_half, const double* conv_func,
        size_t num_points, const double* uu, const double* vv,
        const double* ww, double cell_size_rad, double w_scale,
        int grid_size, const double* grid, double* vis);
/* void forms (failures are reported on stderr and by gg_last_error). */
GG_API void oskar_degrid_wproj_f(const size_t num_w_planes,
        const int* support, const int oversample, const int conv_size_half,
        const float* conv_func, const size_t num_points, const float* uu,
        const float* vv, const float* ww, const float cell_size_rad,
        const float w_scale, const int grid_size, const float* grid,
        float* vis);
GG_API void oskar_degrid_wproj_d(const size_t num_w_planes,
        const int* support, const int oversample, const int conv_size_half,
        const double* conv_func, const size_t num_points, const double* uu,
        const double* vv, const double* ww, const double cell_size_rad,
        const double w_scale, const int grid_size, const double* grid,
        double* vis);

/* ---------------------------------------------------------------------- */
/* Uniform weighting                                                      */
/* ---------------------------------------------------------------------- */

/* Same prototypes and semantics as the reference's uniform-weighting
 * functions (utils/oskar_grid_weights.h:60-144, oskar_grid_weights.c:
 * 38-172), which the reference runs before gridding (main.cpp:230-286):
 *   write: grid[gv][gu] += weight[i] for every point on the grid (a real
 *          grid_size^2 density grid, accumulated), *num_skipped = points
 *          off the grid;
 *   read:  weight_out[i] = weight_in[i] / grid[gv][gu] (0 where the
 *          density is 0) for points on the grid; off-grid points leave
 *          weight_out untouched; *num_skipped set.
 * with gu = (int)round(-uu * grid_size * cell_size_rad) + grid_size / 2
 * and gv likewise from vv, in the call's precision.  Results are
 * bit-identical to the reference's serial code: each cell's weights are
 * added in point order.  Host pointers, synchronous. */
GG_API void oskar_grid_weights_write_f(const size_t num_points,
        const float* uu, const float* vv, const float* weight,
        const float cell_size_rad, const int grid_size, size_t* num_skipped,
        float* grid);
GG_API void oskar_grid_weights_write_d(const size_t num_points,
        const double* uu, const double* vv, const double* weight,
        const double cell_size_rad, const int grid_size, size_t* num_skipped,
        double* grid);
GG_API void oskar_grid_weights_read_f(const size_t num_points,
        const float* uu, const float* vv, const float* weight_in,
        float* weight_out, const float cell_size_rad, const int grid_size,
        size_t* num_skipped, const float* grid);
GG_API void oskar_grid_weights_read_d(const size_t num_points,
        const double* uu, const double* vv, const double* weight_in,
        double* weight_out, const double cell_size_rad, const int grid_size,
        size_t* num_skipped, const double* grid);
/* Status-returning forms (same arguments). */
GG_API int gg_grid_weights_write_f(size_t num_points, const float* uu,
        const float* vv, const float* weight, float cell_size_rad,
        int grid_size, size_t* num_skipped, float* grid);
GG_API int gg_grid_weights_write_d(size_t num_points, const double* uu,
        const double* vv, const double* weight, double cell_size_rad,
        int grid_size, size_t* num_skipped, double* grid);
GG_API int gg_grid_weights_read_f(size_t num_points, const float* uu,
        const float* vv, const float* weight_in, float* weight_out,
        float cell_size_rad, int grid_size, size_t* num_skipped,
        const float* grid);
GG_API int gg_grid_weights_read_d(size_t num_points, const double* uu,
        const double* vv, const double* weight_in, double* weight_out,
        double cell_size_rad, int grid_size, size_t* num_skipped,
        const double* grid);
/* Device-pointer forms on a stream: *d_num_skipped (64-bit) is set, the
 * density grid accumulated.  The write form uses the plan's sort
 * workspace (and discards geometry kept for a batched replay). */
GG_API int gg_grid_weights_write_f_device(gg_plan* plan, size_t num_points,
        const float* d_uu, const float* d_vv, const float* d_weight,
        float cell_size_rad, int grid_size, unsigned long long* d_num_skipped,
        float* d_grid, void* stream);
GG_API int gg_grid_weights_write_d_device(gg_plan* plan, size_t num_points,
        const double* d_uu, const double* d_vv, const double* d_weight,
        double cell_size_rad, int grid_size,
        unsigned long long* d_num_skipped, double* d_grid, void* stream);
GG_API int gg_grid_weights_read_f_device(gg_plan* plan, size_t num_points,
        const float* d_uu, const float* d_vv, const float* d_weight_in,
        float* d_weight_out, float cell_size_rad, int grid_size,
        unsigned long long* d_num_skipped, const float* d_grid, void* stream);
GG_API int gg_grid_weights_read_d_device(gg_plan* plan, size_t num_points,
        const double* d_uu, const double* d_vv, const double* d_weight_in,
        double* d_weight_out, double cell_size_rad, int grid_size,
        unsigned long long* d_num_skipped, const double* d_grid,
        void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GPUGRID_H_ */
