/*
 * dvc_gpu.h — C ABI of the GB300 digital-volume-correlation engine
 * (libdvcgpu.so). Plain C types only: caller-owned host (or device) buffers,
 * status integers, no exceptions and no C++/torch types across the boundary.
 *
 * The reference (TomographicImaging/DigitalVolumeCorrelation) has no library
 * API: its hot path is the C++ class seam Search::process_point
 * (Core/Search.cpp:95-192), called serially by the `dvc` executable
 * (Core/dvc.cpp:233-303), signalling results by throwing Point_Good /
 * Range_Fail / Convg_Fail (Core/Utility.h:76-79). Each entry point below
 * names the reference function it replaces. Function-level entry points
 * (interpolation, objective, strain) exist so each reference function can be
 * checked on its own against the FP64 oracle.
 *
 * Error convention: every function returns DVC_OK (0) or a negative DVC_E_*
 * code; dvc_gpu_last_error() returns a message for the calling thread.
 * Per-point search results use the reference's status integers
 * (Core/Utility.h:38-41).
 */
#ifndef DVC_GPU_H
#define DVC_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DVC_ABI_VERSION 3

/* per-point status, identical to Core/Utility.h:38-41 */
#define DVC_POINT_GOOD 0
#define DVC_RANGE_FAIL (-1)
#define DVC_CONVG_FAIL (-2)
#define DVC_NOT_SEARCH (-3)

/* return codes */
#define DVC_OK 0
#define DVC_E_ARG (-10)      /* invalid argument (sizes, enums, limits)        */
#define DVC_E_CUDA (-11)     /* CUDA runtime error                              */
#define DVC_E_NOMEM (-12)    /* device allocation failed                        */
#define DVC_E_TIMEOUT (-13)  /* a bounded device-side wait gave up              */
#define DVC_E_RANGE (-14)    /* interpolation request outside the active box    */

/* enums: same numbering as the reference's (Core/Utility.h:51-88) */
enum dvc_objfcn { DVC_SAD = 0, DVC_SSD = 1, DVC_ZSSD = 2, DVC_NSSD = 3, DVC_ZNSSD = 4 };
enum dvc_interp { DVC_NEAREST = 0, DVC_TRILINEAR = 1, DVC_TRICUBIC = 2 };
enum dvc_geom { DVC_CUBE = 0, DVC_SPHERE = 1 };

/* how each point's starting translation is chosen */
enum dvc_seed_mode {
  /* reference semantics (Core/Search.cpp:277-377): mean (u,v,w) of the
     already-processed good points among the point's neighbour list, else
     rigid_trans. Points run in `order`; a point waits for the neighbours
     that precede it. */
  DVC_SEED_NEIGHBOURS = 0,
  /* caller supplies one (u,v,w) seed per point; points are independent */
  DVC_SEED_GIVEN = 1,
  /* every point starts from rigid_trans; points are independent */
  DVC_SEED_RIGID = 2,
  /* caller supplies all 12 start parameters per point (u v w phi the psi exx
     eyy ezz exy eyz exz, the first num_srch_dof used): the start estimate and
     the coarse grid are skipped, Gauss-Newton starts there. The learned
     proposer's mode (dvc_gpu_process_learned); points are independent. */
  DVC_SEED_PARAMS = 3
};

/* The search's coarse stage and refinement. The reference's process_point
   runs trgrid_global then min_Lev_Mar (Core/Search.cpp:132,141); its source
   also holds two alternatives that no input key selects: random_global
   (:1045-1098; as many random translations as the grid has points, from a
   clock-seeded rand(), each component uniform in [-disp_max, disp_max))
   and Nelder-Mead through look_with(amoeba, ...) (:150-181, 379-440,
   680-932; Convg_Fail after 2000 evaluations). Here they are opt-in. */
enum dvc_coarse { DVC_COARSE_GRID = 0, DVC_COARSE_RANDOM = 1 };
enum dvc_refine { DVC_REFINE_GAUSS_NEWTON = 0, DVC_REFINE_NELDER_MEAD = 1 };

/* Search configuration: the `dvc` input-file keys that shape the hot path
   (Core/Utility.h:90-134 RunControl; limits Core/InputRead.cpp:519-631). */
typedef struct dvc_params {
  int vol_wide, vol_high, vol_tall; /* voxels; x fastest, then y, then z      */
  int bytes_per_voxel;              /* 1 (uint8) or 2 (uint16, native endian) */
  int subvol_geom;                  /* dvc_geom                               */
  int subvol_size;                  /* cube side / sphere diameter, voxels    */
  int subvol_npts;                  /* 1..50000                               */
  double subvol_aspect[3];          /* default 1 1 1                          */
  int disp_max;                     /* voxels                                 */
  int num_srch_dof;                 /* 3, 6 or 12                             */
  int obj_function;                 /* dvc_objfcn                             */
  int interp_type;                  /* dvc_interp                             */
  double basin_radius;              /* 0 = no coarse grid search              */
  double rigid_trans[3];            /* default 0 0 0                          */
  unsigned int sphere_seed;         /* mt19937 seed of sphere subvolumes; the
                                       reference's reproducible test mode uses 1
                                       (Core/Search.cpp:102-105)               */
  /* subvolume pre-check (keywords subvol_thresh, gray_thresh_min/max,
     min_vol_fract; Core/InputRead.cpp:282-323, limits :564-571): with
     subvol_thresh = 1 a point whose reference samples lie in
     [gray_thresh_min, gray_thresh_max] for less than min_vol_fract of the
     samples is not searched (DVC_NOT_SEARCH). The reference parses and
     echoes these keywords but its search never applies them; 0 keeps its
     behaviour. */
  int subvol_thresh;
  double gray_thresh_min, gray_thresh_max; /* 0 <= min < max <= 2^(8*bytes_per_voxel) */
  double min_vol_fract;                    /* 0..1 */
  /* search stages (no input key in the reference; 0 = its defaults) */
  int coarse_method;          /* dvc_coarse: with basin_radius > 0, the grid or
                                 random_global's translations                */
  int refine_method;          /* dvc_refine: Gauss-Newton or Nelder-Mead     */
  unsigned int coarse_seed;   /* srand() seed of random_global's draws (the
                                 reference uses the clock, time(NULL))        */
} dvc_params;

/* Run statistics returned by dvc_gpu_process. */
typedef struct dvc_stats {
  int n_processed;        /* points searched                                   */
  int n_good, n_range_fail, n_convg_fail;
  long long n_evaluations; /* objective evaluations (grid + GN + ref + final)  */
  long long n_gn_iterations;
  double kernel_ms;       /* device time of the search launch (CUDA events)    */
  double total_ms;        /* wall time of the call                             */
} dvc_stats;

typedef struct dvc_engine dvc_engine; /* opaque: device state for one volume pair */

/* ---- library ------------------------------------------------------------ */
const char *dvc_gpu_version(void);
const char *dvc_gpu_last_error(void);
int dvc_gpu_abi_version(void);

/* ---- engine: both volumes resident in HBM -------------------------------
 * Replaces Search::Search (Core/Search.cpp:24-82) plus the per-point volume
 * reads of Interpolate::kernels (Core/Interpolate.cpp:144-258): the reference
 * re-reads two est_box regions from disk for every point; here each volume is
 * uploaded once. `ref_vox`/`cor_vox` are host buffers of
 * vol_wide*vol_high*vol_tall voxels (header already skipped). For 16-bit data
 * `big_endian` != 0 byte-swaps on upload (Core/Interpolate.cpp:233-242). */
int dvc_gpu_create(dvc_engine **out, const dvc_params *p, const void *ref_vox,
                   const void *cor_vox, int big_endian);
/* Same, for volumes already in device memory (the engine keeps the pointers;
   the caller keeps the buffers alive). Each buffer must be readable for 64
   bytes past its last voxel (aligned row loads over-read the end). */
int dvc_gpu_create_device(dvc_engine **out, const dvc_params *p, const void *ref_vox_dev,
                          const void *cor_vox_dev);
void dvc_gpu_destroy(dvc_engine *e);

/* ---- the search: Search::process_point for many points ------------------
 * Replaces the serial loop of Core/dvc.cpp:233-303 over
 * Search::process_point (Core/Search.cpp:95-192): per point the reference
 * subvolume interpolation, the start estimate (starting_param), the coarse
 * translation grid (trgrid_global, :934-1043), the Gauss-Newton refinement
 * (min_Lev_Mar, :194-246) and the final objective (:187).
 *   points    [n_points*3] x,y,z of every ROI point (host)
 *   order     [n_process]  indices into points, processing order (host)
 *   neigh     [n_points*n_neigh] neighbour indices incl. self (host); used by
 *             DVC_SEED_NEIGHBOURS, may be NULL otherwise
 *   seeds     [n_points*3] starting (u,v,w) for DVC_SEED_GIVEN, else NULL
 * outputs, indexed by point (entries of points never processed are set to
 * DVC_NOT_SEARCH / 0):
 *   status    [n_points]   DVC_POINT_GOOD / DVC_RANGE_FAIL
 *   objmin    [n_points]   objective at the optimum (0 when not good)
 *   params    [n_points*12] u v w phi the psi exx eyy ezz exy eyz exz (first
 *             num_srch_dof valid, rest 0; zeros when not good)
 *   gn_iters  [n_points] Gauss-Newton iterations taken (may be NULL)
 *   stats     may be NULL */
int dvc_gpu_process(dvc_engine *e, int n_points, const double *points, int n_process,
                    const int *order, int n_neigh, const int *neigh, int seed_mode,
                    const double *seeds, int *status, double *objmin, double *params,
                    int *gn_iters, dvc_stats *stats);

/* Same as dvc_gpu_process with every array already in device memory
   (points, order, neigh, seeds; outputs status, objmin, params, gn_iters).
   Enqueued on `stream` (cudaStream_t, may be NULL); returns once enqueued;
   stats are not filled. Errors found on the device (a bounded wait that gave
   up) are read afterwards with dvc_gpu_last_status. */
int dvc_gpu_process_device(dvc_engine *e, int n_points, const double *points_dev, int n_process,
                           const int *order_dev, int n_neigh, const int *neigh_dev, int seed_mode,
                           const double *seeds_dev, int *status_dev, double *objmin_dev,
                           double *params_dev, int *gn_iters_dev, void *stream);

/* Outcome on the device of this engine's most recent search launch (any of
   the search calls, the plan calls that use this engine's workspace, and the
   allocation-free call while no later call on any engine reused its array);
   waits for the device first. The reference surfaces every failure as an
   exception or a status (Core/Utility.h:76-86); a device launch cannot throw,
   so it records the first failure in a flag that this reads:
   DVC_OK; DVC_E_TIMEOUT when a bounded wait gave up (a neighbour's result or
   a ready-queue slot that did not arrive within the wait limit: those points
   are left DVC_NOT_SEARCH; or a shared-memory staging copy that did not land:
   the CTA then evaluated from global memory, results unchanged); DVC_E_ARG
   when a plan's point named no configuration. dvc_gpu_process and the other
   host-array calls return the same code themselves. */
int dvc_gpu_last_status(dvc_engine *e);

/* Polls a dependency wait of this engine's searches makes before it gives up
   (a point waiting for a neighbour's result, a cluster waiting for a
   ready-queue slot): polls >= 0 sets the bound, a negative value restores the
   default (2^25 polls, about 4 s per wait). The reference waits on nothing
   (one host thread runs the points in order); the bound keeps every device
   wait finite, and a small one lets a test make a wait run out. */
int dvc_gpu_set_wait_limit(dvc_engine *e, long long polls);

/* ---- volume files -------------------------------------------------------
 * The reference reads the raw volume files piecewise for every point (one
 * seekg + read per row of the interpolation box, Interpolate::kernels,
 * Core/Interpolate.cpp:144-258; endian swap on the host, :219-250). These
 * stream each file once into device memory in 64 MiB chunks through two
 * pinned buffers (file read overlapping the copy), swapping big-endian
 * 16-bit data on the device. */
typedef struct dvc_volume_info {
  int nx, ny, nz;          /* DimSize */
  int bytes_per_voxel;     /* 1 (MET_UCHAR/MET_CHAR) or 2 (MET_USHORT/MET_SHORT) */
  int big_endian;          /* BinaryDataByteOrderMSB / ElementByteOrderMSB (16-bit) */
  long long header_bytes;  /* bytes to skip in data_file (HeaderSize; LOCAL data) */
  char data_file[1024];    /* ElementDataFile, relative to the .mhd's folder */
} dvc_volume_info;
/* Reads a MetaImage (.mhd) header: NDims 3, DimSize, ElementType (8 or
   16 bit), HeaderSize, byte order, ElementDataFile (a file name or LOCAL);
   host code, no GPU call. The reference takes the same facts from input-file
   keys (vol_wide/high/tall, vol_bit_depth, vol_hdr_lngth, vol_endian). */
int dvc_gpu_read_mhd(const char *mhd_path, dvc_volume_info *out);
/* Streams nx*ny*nz voxels from `path` (after header_bytes) into vol_dev on
   `stream`; returns when the volume is in place. */
int dvc_gpu_load_raw(void *vol_dev, const char *path, long long header_bytes, int nx, int ny,
                     int nz, int bytes_per_voxel, int big_endian, void *stream);
/* dvc_gpu_create with both volumes read straight from their files (same
   header length and byte order for both, as the reference's input file has
   one vol_hdr_lngth and one vol_endian). */
int dvc_gpu_create_from_files(dvc_engine **out, const dvc_params *p, const char *ref_path,
                              const char *cor_path, long long header_bytes, int big_endian);

/* ---- allocation-free search ---------------------------------------------
 * No counterpart in the reference. Same as dvc_gpu_process_device, but the
 * call allocates no device memory and calls no allocating routine: its scratch
 * (per-point done flags and ranks, work counter, evaluation counters) is a
 * fixed array inside the library, sized for DVC_NOALLOC_MAX_POINTS points,
 * that every GPU using the library keeps until the process exits. For callers
 * that must not allocate while they search (a host program that hands out all
 * device memory from its own pool, or one recording its work where device
 * allocation is not allowed). More points than DVC_NOALLOC_MAX_POINTS are
 * rejected with DVC_E_ARG. The first call on a device looks up the array's
 * device address (and may load the library's device code): make that first
 * call before any stream capture. All calls share the one array; calls whose
 * work overlaps on the GPU race on it, so serialise them. The engine must
 * already exist (dvc_gpu_create / dvc_gpu_create_device allocate).
 * dvc_gpu_last_counters and dvc_gpu_last_status report the call until the
 * next allocation-free call (from any engine) overwrites the array. */
#define DVC_NOALLOC_MAX_POINTS 65536
int dvc_gpu_process_device_noalloc(dvc_engine *e, int n_points, const double *points_dev,
                                   int n_process, const int *order_dev, int n_neigh,
                                   const int *neigh_dev, int seed_mode, const double *seeds_dev,
                                   int *status_dev, double *objmin_dev, double *params_dev,
                                   int *gn_iters_dev, void *stream);

/* CTAs per point (one cluster) for this engine's searches: 1, 2, 4 or 8, or
   0 (the default, or the DVC_CLUSTER environment variable at creation) to
   choose per call from the sample count and seeding. A width whose staging
   box or sample state does not fit is widened. The search's results depend
   on the width only through FP32/FP64 summation order. No counterpart in
   the reference (one thread per point). */
int dvc_gpu_set_cluster(dvc_engine *e, int cluster);
/* Shape of this engine's most recent search launch: out[0] CTAs per point,
   out[1] CTAs in the grid, out[2] staging of the correlate region (0 none,
   1 one box covering every grid translation, 2 one box per z slab of
   translations), out[3] dynamic shared memory per CTA in bytes. */
int dvc_gpu_last_launch(dvc_engine *e, int out[4]);

/* Rank windows of this engine's most recent search with the reference's
   seeding (dataflow scheduled, cluster width chosen by the engine): the
   ranks [0, out[0]) and [out[1], n_process) were searched by launches of
   out[2] CTAs per point, the ranks between them at out[0] of
   dvc_gpu_last_launch. out[0] = out[1] = n_process: one launch. Each window
   is a launch of its own after the previous one (a point's predecessors in
   an earlier window have finished); a point's cluster width follows from its
   rank alone, so results do not depend on timing. */
int dvc_gpu_last_windows(dvc_engine *e, int out[3]);

/* Counters of the most recent dvc_gpu_process / dvc_gpu_process_device call
   on this engine (waits for it to finish): out[0] objective evaluations
   (reference subvolume, grid offsets, Gauss-Newton evaluations, final
   objective), out[1] Gauss-Newton iterations, out[2] sample evaluations that
   fell in the interpolation box's last cell plane, which the reference leaves
   undefined. The reference reports run counts only as pt/sec and status
   percentages in its .stat file (Core/dvc.cpp:322-338). */
int dvc_gpu_last_counters(dvc_engine *e, long long out[3]);

/* Diagnostics of the same call: SM clock cycles spent per phase of the
   per-point loop, summed over every CTA of the launch: out[0] taking work and
   forming the start estimate (neighbour waits included), out[1] reference
   subvolume and sample setup, out[2] coarse translation grid, out[3]
   Gauss-Newton set-up and exit, out[4] final objective and result; per
   Gauss-Newton iteration out[5] warp matrices, out[6] range check and
   staging, out[7] sample evaluation, out[8] reductions, out[9] assembly,
   solve and update, out[10] the G'G accumulation of the evaluations. No
   counterpart in the reference (it has no per-phase timing). */
#define DVC_N_PHASES 11
int dvc_gpu_last_phase_cycles(dvc_engine *e, long long out[DVC_N_PHASES]);

/* ---- several search configurations in one launch -------------------------
 * The reference runs one configuration per `dvc` run: every point of the
 * cloud is searched by Search::process_point (Core/Search.cpp:95-192) with the
 * run's one RunControl (Core/dvc.cpp:233-303). A plan holds several
 * configurations, each an engine from dvc_gpu_create / dvc_gpu_create_device
 * (its dvc_params: subvolume geometry, size and sample count, search degrees
 * of freedom, objective, grid), all on the same volumes (the same ref and
 * correlate buffers, dimensions, voxel type and interpolation). Each point
 * names its configuration; one persistent launch searches every point, its
 * clusters taking the next point from the work queue whatever its
 * configuration, and each point's result is the one its configuration's own
 * engine would give at the same cluster width. The engines must outlive the
 * plan; the plan's calls use the first engine's workspace and counters
 * (dvc_gpu_last_counters on configs[0]).
 *   cluster   CTAs per point (1, 2, 4 or 8), or 0 to choose from the sample
 *             counts; every configuration must fit the shared memory of a
 *             CTA at that width (DVC_E_ARG otherwise) */
typedef struct dvc_plan dvc_plan;
int dvc_gpu_plan_create(dvc_plan **out, dvc_engine *const *configs, int n_configs, int cluster);
void dvc_gpu_plan_destroy(dvc_plan *plan);
/* The plan's launch shape: CTAs per point, whether the correlate volume is
   staged in shared memory (TMA) for the configurations whose box fits, how
   many configurations are staged, dynamic shared memory per CTA. */
int dvc_gpu_plan_info(const dvc_plan *plan, int *cluster, int *staging, int *n_staged,
                      long long *smem_bytes);
/* Rebuild the plan at another launch shape (cluster 1, 2, 4 or 8; staging 0
   or 1). Waits for the device first. */
int dvc_gpu_plan_set_shape(dvc_plan *plan, int cluster, int staging);
/* Search with point_cfg[i] in 0..n_configs-1 the configuration of point i;
   every other argument as dvc_gpu_process_device. Enqueued on `stream`. A
   point whose configuration index is out of range is left unsearched
   (DVC_NOT_SEARCH) and the launch's error flag records DVC_E_ARG. The first
   call with a given point count may grow the workspace (a device
   allocation): make it before capturing later calls in a CUDA graph. */
int dvc_gpu_plan_process_device(dvc_plan *plan, const int *point_cfg_dev, int n_points,
                                const double *points_dev, int n_process, const int *order_dev,
                                int n_neigh, const int *neigh_dev, int seed_mode,
                                const double *seeds_dev, int *status_dev, double *objmin_dev,
                                double *params_dev, int *gn_iters_dev, void *stream);
/* Same with host arrays (copied in and out; blocking), as dvc_gpu_process. */
int dvc_gpu_plan_process(dvc_plan *plan, const int *point_cfg, int n_points, const double *points,
                         int n_process, const int *order, int n_neigh, const int *neigh,
                         int seed_mode, const double *seeds, int *status, double *objmin,
                         double *params, int *gn_iters, dvc_stats *stats);
/* Autotuner (no counterpart in the reference): times the plan's search over
   the given points (device arrays, as dvc_gpu_plan_process_device; outputs
   are scratch) at every launch shape that fits: cluster widths 1, 2, 4, 8,
   each with and without staging. Each shape runs `reps` timed launches
   after one untimed one; the fastest shape (least mean time) is kept.
   ms_out[2*j + s] (may be NULL; 8 entries) gets the mean milliseconds of width
   2^j with staging s, or -1 for a shape that does not fit. Blocking. */
int dvc_gpu_plan_autotune(dvc_plan *plan, const int *point_cfg_dev, int n_points,
                          const double *points_dev, int n_process, const int *order_dev,
                          int n_neigh, const int *neigh_dev, int seed_mode,
                          const double *seeds_dev, int *status_dev, double *objmin_dev,
                          double *params_dev, int reps, double ms_out[8]);

/* ---- learned initial guess (no counterpart in the reference) ------------
 * A small 3D CNN proposes each point's start parameters from its reference
 * and correlate patches (32^3 voxels centred on the point, each normalised to
 * zero mean and unit variance), in place of Search::starting_param and
 * trgrid_global (Core/Search.cpp:277-377,934-1043). Conv 2->16->32->64->96
 * (3^3, stride 2, ReLU), dense 768->128 (ReLU) ->12; outputs are the
 * parameters divided by fixed scales (translations 10 voxels, rotations
 * 0.05 rad, strains 0.02). FP32 master weights; the convolutions run on the
 * tensor cores with BF16 operands and FP32 accumulation (environment variable
 * DVC_CNN_FP32=1: on the FP32 pipes, FP32 operands); training by mean squared
 * error and Adam, all on the GPU. */
typedef struct dvc_cnn dvc_cnn;
int dvc_cnn_create(dvc_cnn **out, unsigned seed);  /* He-normal initial weights */
void dvc_cnn_destroy(dvc_cnn *net);
int dvc_cnn_param_count(void);
int dvc_cnn_get_weights(dvc_cnn *net, float *host, int n);
int dvc_cnn_set_weights(dvc_cnn *net, const float *host, int n); /* resets the optimizer */
/* patches of points idx[0..n) (all points if idx is NULL) of the engine's
   volume pair: patches_dev [n][2][32][32][32] FP32 (reference, correlate) */
int dvc_cnn_patches(dvc_engine *e, int n, const double *points_dev, const int *idx_dev,
                    float *patches_dev, void *stream);
/* network outputs (scaled parameters) [batch][12] */
int dvc_cnn_forward(dvc_cnn *net, int batch, const float *patches_dev, float *out_dev, void *stream);
/* loss (mean squared error of the scaled outputs against targets [batch][12],
   raw parameters, FP32) and its gradient w.r.t. every weight (grad_host may be
   NULL); no update */
int dvc_cnn_gradients(dvc_cnn *net, int batch, const float *patches_dev, const float *targets_dev,
                      float *grad_host, float *loss);
/* one Adam step (beta 0.9 / 0.999, eps 1e-8) at learning rate lr */
int dvc_cnn_train_step(dvc_cnn *net, int batch, const float *patches_dev, const float *targets_dev,
                       float lr, float *loss);
/* The learned search: the network's start parameters for every point in
   `order`, Gauss-Newton from there (DVC_SEED_PARAMS), then, for the points
   whose search failed or whose objective exceeds obj_threshold, the plain
   search (coarse grid + Gauss-Newton) seeded with the network's translation.
   Device arrays as in dvc_gpu_process_device; *n_fallback (host) receives the
   number of points searched again. The points are taken in locality order
   (sorted by the Morton code of their cell) for the network passes and the
   searches; every point's result is independent of the order given.
   Synchronises the stream; dvc_gpu_last_counters then reports the sum over
   both searches. */
int dvc_gpu_process_learned(dvc_engine *e, dvc_cnn *net, int n_points, const double *points_dev,
                            int n_process, const int *order_dev, double obj_threshold,
                            int *status_dev, double *objmin_dev, double *params_dev,
                            int *gn_iters_dev, int *n_fallback, void *stream);

/* ---- processing order and neighbours on the GPU --------------------------
 * DataCloud::sort_order_neighbors (Core/DataCloud.cpp:69-144): order[n] the
 * points by distance from `start`, neigh[n * min(k, n)] each point's k
 * nearest (itself first), distances bit-identical to the reference's, ties by
 * point index (the reference's std::sort leaves ties in an order of its own).
 * Host arrays. */
int dvc_gpu_order_neighbours(int n, const double *points, const double start[3], int k, int *order,
                             int *neigh);

/* ---- function-level entry points ----------------------------------------
 * Interpolate one volume (0 = reference, 1 = correlate) at n points, with the
 * interpolation box of this engine's search (Search::Search est_box_nom,
 * Core/Search.cpp:66-80) centred on `center` (Interpolate::center_on,
 * Core/Interpolate.cpp:569-574). Replaces Interpolate::nearest / tri_lin /
 * tri_cub_Lek (Core/Interpolate.cpp:404-567). Returns DVC_E_RANGE when the
 * points' bounding box leaves the active box (the reference's Intrp_Fail,
 * Core/Interpolate.cpp:474-481); `out` is then untouched. */
int dvc_gpu_interpolate(dvc_engine *e, int volume, const double center[3], int n,
                        const double *pts, int interp_type, double *out);

/* Objective of two sample vectors, with optional residual vector. Replaces
   obj_SAD .. obj_ZNSSD (Core/ObjectiveFunctions.cpp:24-263). */
int dvc_gpu_objective(int obj_function, int n, const double *ref, const double *tar,
                      double *obj, double *residual);

/* Strain-window least-squares fit for every point. Replaces the per-point
 * loop of the `strain` executable (Core/strain.cpp:402-591).
 *   pts [n*3], status [n], objmin [n], disp [n*3]  (from the .disp file)
 *   neigh [n*n_neigh]                               (from the .sort.csv file)
 *   ndp strain window (already clamped by the caller as Core/strain.cpp:204-207)
 *   objt objmin threshold, refill (-r), planar: bit0 yz_only, bit1 zx_only,
 *   bit2 xy_only (Core/strain.cpp:340-370)
 * outputs: u_fit [n*3], pts_in_sw [n], sw_radius [n], e_strain [n*9],
 *   l_strain [n*9] (exx eyy ezz exy eyz exz p1 p2 p3), dgrad [n*9] row-major */
int dvc_gpu_strain(int n, const double *pts, const int *status, const double *objmin,
                   const double *disp, int n_neigh, const int *neigh, int ndp, double objt,
                   int refill, int planar, double *u_fit, int *pts_in_sw, double *sw_radius,
                   double *e_strain, double *l_strain, double *dgrad);

/* Synthetic speckle volume for benchmarks and tests (no reference
   counterpart): Gaussian blobs rendered at the inverse-deformed position of
   every voxel plus Gaussian noise, clipped and rounded to uint8/uint16.
   `deform` selects the field: 0 none; 1 affine u(X) = t + E (X - c) with
   coef = {t0,t1,t2, E00..E22 (9), c0,c1,c2}; 2 sinusoid u_i = A sin(2 pi X_j / L)
   with coef = {A, L}; 3 affine plus Gaussian bumps, coef = {t (3), E (9),
   c (3), n, n x (p (3), s, a (3))}, u = t + E (X - c) + sum a exp(-|X - p|^2 /
   (2 s^2)), n <= 32; 4 two affine pieces split by the plane X_x = split,
   coef = {t1 (3), E1 (9), c1 (3), t2 (3), E2 (9), c2 (3), split} (blob
   amplitudes >= 0); 5 bending and jump, coef = {kappa, xc, h, J, z0, w}:
   u_x = (J/2) tanh((X_z - z0)/w), u_y = 0, u_z = (kappa/2)((X_x - xc)^2 - h).
   vol_dev is a device buffer; blobs a host array. */
int dvc_gpu_synth_volume(void *vol_dev, int nx, int ny, int nz, int bytes_per_voxel,
                         int n_blobs, const float *blobs /* host, n_blobs*5: x y z sigma amp */,
                         int deform, const double *coef, float background, float noise_sigma,
                         unsigned long long noise_seed, float vmax, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* DVC_GPU_H */
