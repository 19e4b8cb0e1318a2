/*
 * pvdb.h — C ABI of libpvdb, the GB300 (sm_103a) implementation of PlenVDB's
 * differentiable sparse-grid ray-marching path.
 *
 * Every entry point:
 *   - returns an int status (PVDB_OK on success; see PVDB_ERR_*); the message of
 *     the last failure on the calling thread is available from pvdb_last_error();
 *   - takes plain pointers and sizes only (no framework types);
 *   - takes an explicit stream (a cudaStream_t passed as void*; NULL = legacy
 *     default stream) and never synchronises unless its comment says so;
 *   - where a buffer argument carries a `mem` flag, PVDB_MEM_HOST means a host
 *     buffer that the call copies to/from the device itself (and then
 *     synchronises the stream before returning, like the reference's pybind
 *     calls), PVDB_MEM_DEVICE means a device buffer used in place.
 *
 * Reference interfaces cited below are paths inside wolfball/PlenVDB.
 */
#ifndef PVDB_H
#define PVDB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PVDB_OK 0
#define PVDB_ERR_ARG 1      /* bad pointer, size, shape or mode */
#define PVDB_ERR_CUDA 2     /* a CUDA runtime call or kernel launch failed */
#define PVDB_ERR_TIMEOUT 3  /* a bounded device-side wait gave up */
#define PVDB_ERR_NOMEM 4    /* device or host allocation failed */
#define PVDB_ERR_STATE 5    /* object not in a state that allows the call */
#define PVDB_ERR_IO 6       /* file missing, truncated or failing its checksum */

#define PVDB_MEM_HOST 0
#define PVDB_MEM_DEVICE 1

#define PVDB_WHICH_DATA 0
#define PVDB_WHICH_GRAD 1

typedef struct pvdb_grid_s* pvdb_grid;
typedef struct pvdb_opt_s* pvdb_opt;
typedef struct pvdb_march_s* pvdb_march;
typedef struct pvdb_renderer_s* pvdb_renderer;
typedef void* pvdb_stream; /* cudaStream_t */

/* ---------------------------------------------------------------- library */

/* Version string of the library. */
const char* pvdb_version(void);

/* Copies the last error message of the calling thread into buf (NUL-terminated,
 * truncated to len). Returns the status code of that error (PVDB_OK if none). */
int pvdb_last_error(char* buf, size_t len);

/* Test hook: makes the next `count` device allocations made by the library fail
 * with PVDB_ERR_NOMEM (host-side injection; no device call is made for them). */
int pvdb_debug_fail_next_allocs(int count);
/* Test hook of the bounded device-side waits (no counterpart in the
 * reference): spins > 0 replaces the built-in spin limit of the device waits
 * (radix sort and march look-backs, tensor-core MMA waits, leaf-staging copy
 * waits; 0 restores it); hold_first == 1 makes the first publisher of each
 * look-back chain (and the rgbnet backward's MMA issuer) withhold its work, so
 * that the waits behind it run out and the call reports PVDB_ERR_TIMEOUT;
 * hold_first == 2 makes the first block of the staged density pass
 * (pvdb_march_set_leaf_staging) issue no leaf copies, so its copy wait runs
 * out (it then reads global memory: the results are unchanged, the workspace
 * reports PVDB_ERR_TIMEOUT). Applies to launches made after the call (a
 * captured train-step graph keeps the values it was captured with). */
int pvdb_debug_wait_limit(uint32_t spins, int32_t hold_first);
/* Test hook (no counterpart in the reference): blocks = 2 or 3 forces the
 * resident-blocks-per-SM variant of the BF16 train step's k0 gather (one
 * source compiled for 128 or 80 registers a thread; the library takes 2 for
 * batches up to 32768 rays and 3 above), 0 restores that choice. Both give
 * bitwise identical results. Applies to launches made after the call (a
 * captured train-step graph keeps the variant it was captured with). */
int pvdb_debug_k0_blocks(int blocks);

/* Stage profiler. Between begin and end, pvdb_train_step and
 * pvdb_renderer_render record CUDA events on their stream at stage boundaries
 * (up to max_steps calls, no synchronisation). end synchronises on those events
 * and writes, for each mark i < n_marks, the total milliseconds between the
 * previous recorded mark and mark i, summed over the calls. Train-step marks:
 * 1 march forward, 2 k0 gather, 3 rgbnet forward, 4 composite + loss,
 * 5 rgbnet backward, 6 march backward (keys), 7 grouping by cell, 8 per-voxel
 * sums, 9 TV, 10 voxel Adam, 11 rgbnet Adam (a profiled step runs these in
 * sequence on its stream). Renderer marks: 1 count march,
 * 2 scan, 3 fill march, 4 rgbnet, 5 composite. */
int pvdb_profile_begin(int32_t max_steps);
/* Number of kernels the library has launched so far (all threads). */
uint64_t pvdb_launch_count(void);
int pvdb_profile_end(float* ms, int32_t n_marks, int32_t* n_calls);

/* ------------------------------------------------------------------ grids
 * A grid is a set of 8^3 leaves over a resolution reso[3], with `channels`
 * float values per voxel (data and gradient), a per-voxel active mask and a
 * background value returned for coordinates outside every allocated leaf.
 * Replaces GridType ScaleGrid/VectorGrid and VDBType DensityVDB/ColorVDB
 * (plenvdb/lib/vdb/plenvdb.h:89-303, :389-602).                          */

/* Dense grid, every voxel of [0,reso) active, values 0 — DensityVDB(reso,1) /
 * ColorVDB(reso,n) constructors (plenvdb.h:434-439, :529-534; ScaleGrid::create
 * plenvdb.h:117-125 denseFill(bbox, 0, active=true)). channels must be 1 or a
 * positive multiple of 3 (plenvdb.h:435, :530). */
int pvdb_grid_create(const int32_t reso[3], int32_t channels, float background, pvdb_grid* out);

/* Sparse grid: a leaf is allocated when it holds at least one voxel with
 * active[x*ry*rz + y*rz + z] != 0; that voxel set is the active mask; every
 * stored value starts at `background`. Stands for loading a sparse .vdb
 * (ScaleGrid::load_from plenvdb.h:126-142). */
int pvdb_grid_create_from_mask(const int32_t reso[3], int32_t channels, float background,
                               const uint8_t* active, int32_t mem, pvdb_grid* out);

/* Same topology, channel count, background and resolution as `like`. */
int pvdb_grid_create_like(pvdb_grid like, int32_t channels, float background, pvdb_grid* out);

int pvdb_grid_destroy(pvdb_grid g);

/* getinfo/getndim (plenvdb.h:401, :423-427); counts are host-side copies. */
int pvdb_grid_get_info(pvdb_grid g, int32_t reso[3], int32_t* channels, int32_t* nleaf,
                       int64_t* nactive, float* background);

/* setReso (plenvdb.h:428). Only changes the resolution used by the dense copies. */
int pvdb_grid_set_reso(pvdb_grid g, int32_t rx, int32_t ry, int32_t rz);

/* copyFromDense (plenvdb.h:149-157, :241-250; densityvdb.cu:31-61,
 * colorvdb.cu:42-77): arr is [rx,ry,rz,channels] row-major; only active voxels
 * are written. which = PVDB_WHICH_DATA or PVDB_WHICH_GRAD (set_grad,
 * plenvdb.h:696). n must equal rx*ry*rz*channels. */
int pvdb_grid_copy_from_dense(pvdb_grid g, int32_t which, const float* arr, int64_t n,
                              int32_t mem, pvdb_stream s);

/* copyToDense / get_dense_grid (plenvdb.h:158-167, :251-267, :408): every voxel
 * of [0,reso) receives its stored value (active or not) or the background. */
int pvdb_grid_copy_to_dense(pvdb_grid g, int32_t which, float* out, int64_t n, int32_t mem,
                            pvdb_stream s);

/* setValuesOn_bymask (plenvdb.h:487-495, densityvdb.cu:64-97): active voxels
 * whose dense mask entry is nonzero get value `val` in every channel. */
int pvdb_grid_set_values_by_mask(pvdb_grid g, const uint8_t* mask, int64_t n, float val,
                                 int32_t mem, pvdb_stream s);

/* forward (plenvdb.h:441-466, :535-556; densityvdb.cu:101-139,
 * colorvdb.cu:81-126): trilinear sample at index-space points (SoA xs,ys,zs),
 * corners outside allocated leaves read the background. out is [n, channels]. */
int pvdb_grid_sample(pvdb_grid g, const float* xs, const float* ys, const float* zs, int64_t n,
                     float* out, int32_t mem, pvdb_stream s);

/* backward (plenvdb.h:468-485, :557-573; densityvdb.cu:16-27, :143-181,
 * colorvdb.cu:28-37, :130-175): adds grad_out[n,channels] x trilinear weight
 * into the gradient of every corner voxel that lies in an allocated leaf (the
 * active mask is ignored, as in the reference). The sum is a deterministic
 * leaf-sorted segmented reduction (bitwise reproducible), not float atomics.
 * The call waits for its stream to finish, as the reference's backward does
 * (plenvdb.h:468-485 ends in a device synchronisation): a bounded wait of the
 * sort that gave up is reported as PVDB_ERR_TIMEOUT, with the gradient left
 * unchanged. */
int pvdb_grid_sample_backward(pvdb_grid g, const float* xs, const float* ys, const float* zs,
                              const float* grad_out, int64_t n, int32_t mem, pvdb_stream s);

/* Same result as pvdb_grid_sample_backward (device buffers only), for callers
 * that cannot let the library allocate device memory: processes that reserve
 * all device memory up front through their own pool or run under a fixed
 * memory budget, and callers that cannot afford the device-wide
 * synchronisation of cudaMalloc/cudaFree. No counterpart in the reference.
 * The call allocates nothing: its scratch is one fixed file-scope device array
 * (about 5.3 MB) that limits a call to n <= 32768 points (PVDB_ERR_ARG beyond
 * that). The array exists on a GPU once the library's module is loaded there
 * and is held until exit; under CUDA's lazy module loading (the default) the
 * first call on a device loads it and looks up its address
 * (cudaGetSymbolAddress), so make that first call before reserving a memory
 * pool or capturing a stream. All calls share the array, so calls that
 * overlap on the GPU (e.g. on two streams) race: serialise them on one stream
 * per device. Like pvdb_grid_sample_backward, the call waits for its stream
 * and reports a sort wait that gave up as PVDB_ERR_TIMEOUT. */
int pvdb_grid_sample_backward_noalloc(pvdb_grid g, const float* xs, const float* ys,
                                      const float* zs, const float* grad_out, int64_t n,
                                      pvdb_stream s);

/* forward_single (plenvdb.h:503-523, densityvdb.cu:376-403,
 * colorvdb.cu:380-413): value at integer coordinates (stored value inside an
 * allocated leaf whether active or not, else background); active_out (may be
 * NULL) receives the active bit (ReadAccessor::isActive, NanoVDB.h:4663-4674). */
int pvdb_grid_lookup(pvdb_grid g, const int32_t* is, const int32_t* js, const int32_t* ks,
                     int64_t n, float* out, uint8_t* active_out, int32_t mem, pvdb_stream s);

/* total_variation_add_grad (plenvdb.h:497-501, :574-578 are stubs in the
 * reference; the math follows lib/cuda/total_variation_kernel.cu:13-67):
 * for each active voxel (every one if dense_mode, else only where the channel's
 * gradient is nonzero) adds sum over the 6 neighbours inside [0,reso) of
 * (w_axis/6)*clamp(v - v_nbr, -1, 1). Neighbour values come from the grid
 * (background outside allocated leaves). mimic_axis_bug != 0 reproduces the
 * reference kernel's use of wz on the x axis (total_variation_kernel.cu:31-32). */
int pvdb_grid_tv_add_grad(pvdb_grid g, float wx, float wy, float wz, int32_t dense_mode,
                          int32_t mimic_axis_bug, pvdb_stream s);

/* Zero the gradient of active voxels (density_zero_grad_kernel
 * densityvdb.cu:353-368, color_zero_grad_kernel colorvdb.cu:355-371). */
int pvdb_grid_zero_grad(pvdb_grid g, pvdb_stream s);

/* Number of leaves in the grid's touched-leaf list as last built (by TV or
 * mode-1 Adam over the leaves a backward touched), 0 if none was built: the
 * leaves whose voxels those passes visit. A measurement aid with no
 * counterpart in the reference; waits for the stream. */
int pvdb_grid_touched_leaves(pvdb_grid g, int64_t* n, pvdb_stream s);

/* Device views of the leaf store (for zero-copy use by a host framework).
 * data/grad: float[nleaf*512*channels] (voxel-major, channel innermost);
 * mask: uint64[nleaf*8]; leaf_table: int32[ldim0*ldim1*ldim2] (-1 = no leaf);
 * leaf_origin: int32[nleaf*3]. Any pointer argument may be NULL. Asking for
 * `data` (or `grad`) marks the values (gradients) as externally written; a
 * caller that keeps the pointer and writes through it again after a later
 * library call must report it with pvdb_grid_mark_written. */
int pvdb_grid_device_views(pvdb_grid g, void** data, void** grad, void** mask,
                           void** leaf_table, void** leaf_origin, int32_t ldim[3]);

/* Report writes through device views: which = PVDB_WHICH_DATA drops the
 * values' derived data (the brick bound, rebuilt by the next march, and the
 * BF16 feature shadow, rebuilt by the next BF16 train step), PVDB_WHICH_GRAD
 * makes every leaf count as possibly holding a gradient. No reference
 * counterpart (the reference copies host arrays in and out on every call). */
int pvdb_grid_mark_written(pvdb_grid g, int32_t which);

/* save_to / load_from (plenvdb.h:143-148, :126-142, :269-276, :211-240).
 * The file holds the leaf topology, active masks, values and a checksum
 * (OpenVDB .vdb I/O is not available; see INTEGRATION notes). Synchronous. */
int pvdb_grid_save(pvdb_grid g, const char* path);
int pvdb_grid_load(const char* path, pvdb_grid* out);

/* ------------------------------------------------------- voxel optimiser
 * Per-voxel Adam over the active voxels of a grid (OptType BaseOptimizer /
 * DensityOpt / ColorOpt, plenvdb.h:686-790; kernels densityvdb.cu:185-349,
 * colorvdb.cu:179-351). Moments are FP32 grids with the grid's topology.     */

int pvdb_opt_create(pvdb_grid g, float lr, float eps, float beta0, float beta1, pvdb_opt* out);
int pvdb_opt_destroy(pvdb_opt o);

/* step(mode) (plenvdb.h:751-767, :774-789): mode 0 plain, 1 skip voxels whose
 * gradient is zero (for multi-channel grids, skip a 3-channel group only when
 * all three are zero, colorvdb.cu:318), 2 per-voxel learning rate. The bias
 * corrected step size is computed on the host in float (plenvdb.h:753).
 * zero_grad_after != 0 clears the gradient of the visited voxels in the same
 * pass (equivalent to calling zero_grad before the next backward). */
int pvdb_opt_step(pvdb_opt o, int32_t mode, int32_t zero_grad_after, pvdb_stream s);

/* zero_grad (plenvdb.h:750, :773). */
int pvdb_opt_zero_grad(pvdb_opt o, pvdb_stream s);

/* set_grad (plenvdb.h:696): dense [rx,ry,rz,channels] into the gradient. */
int pvdb_opt_set_grad(pvdb_opt o, const float* arr, int64_t n, int32_t mem, pvdb_stream s);

/* set_pervoxel_lr (plenvdb.h:713-718): dense [rx,ry,rz] per-voxel lr factors. */
int pvdb_opt_set_pervoxel_lr(pvdb_opt o, const float* count, int64_t n, int32_t mem,
                             pvdb_stream s);

/* update_lr (plenvdb.h:712): lr *= factor. */
int pvdb_opt_update_lr(pvdb_opt o, float factor);

/* get/set Step, Lr, Eps, Beta0, Beta1 (plenvdb.h:697-706). */
int pvdb_opt_get_scalars(pvdb_opt o, int32_t* step, float* lr, float* eps, float* beta0,
                         float* beta1);
int pvdb_opt_set_scalars(pvdb_opt o, int32_t step, float lr, float eps, float beta0, float beta1);

/* The exp_avg / exp_avg_sq moment grids (load_from/save_to plenvdb.h:719-734
 * write them as `prefix`exp_avg.vdb and `prefix`exp_avg_sq.vdb). */
int pvdb_opt_moments(pvdb_opt o, pvdb_grid* exp_avg, pvdb_grid* exp_avg_sq);

/* ------------------------------------------------------------ dense Adam
 * adam_upd / masked_adam_upd / adam_upd_with_perlr (lib/cuda/adam_upd_kernel.cu
 * :8-132, masked_adam.py:128-158) over a flat FP32 parameter buffer (rgbnet).
 * mode 0 plain, 1 skip zero gradients, 2 per-element lr (perlr). All device. */
int pvdb_adam_dense(float* param, const float* grad, float* exp_avg, float* exp_avg_sq,
                    const float* perlr, int64_t n, int32_t step, float beta1, float beta2,
                    float lr, float eps, int32_t mode, pvdb_stream s);

/* ------------------------------------------- DVGO compositing primitives
 * Device buffers only; these mirror render_utils_cuda (lib/cuda/
 * render_utils.cpp:170-184) one for one for the standalone (unfused) path.  */

/* raw2alpha (render_utils_kernel.cu:430-443): exp_d = exp(density+shift),
 * alpha = 1 - (1+exp_d)^(-interval). */
int pvdb_raw2alpha(const float* density, int64_t n, float shift, float interval, float* exp_d,
                   float* alpha, pvdb_stream s);

/* raw2alpha_backward (render_utils_kernel.cu:506-552). */
int pvdb_raw2alpha_backward(const float* exp_d, const float* grad_back, int64_t n,
                            float interval, float* grad, pvdb_stream s);

/* alpha2weight (render_utils_kernel.cu:576-651): points sorted by ray_id
 * (int64, nondecreasing). Writes weight, T [n], alphainv_last [n_rays],
 * i_start, i_end [n_rays] (int64). Early stop once T < 1e-3. */
int pvdb_alpha2weight(const float* alpha, const int64_t* ray_id, int64_t n, int32_t n_rays,
                      float* weight, float* T, float* alphainv_last, int64_t* i_start,
                      int64_t* i_end, pvdb_stream s);

/* alpha2weight_backward (render_utils_kernel.cu:653-707). */
int pvdb_alpha2weight_backward(const float* alpha, const float* weight, const float* T,
                               const float* alphainv_last, const int64_t* i_start,
                               const int64_t* i_end, int32_t n_rays, const float* grad_weights,
                               const float* grad_last, int64_t n, float* grad, pvdb_stream s);

/* sample_pts_on_rays, step 1 (render_utils_kernel.cu:196-242): per ray
 * t_min/t_max and the sample count N_steps = max(ceil((t_max-t_min)|d|/stepdist),1). */
int pvdb_ray_count_samples(const float* rays_o, const float* rays_d, int32_t n_rays,
                           const float xyz_min[3], const float xyz_max[3], float near_,
                           float far_, float stepdist, float* t_min, float* t_max,
                           int64_t* n_steps, pvdb_stream s);

/* sample_pts_on_rays, step 2: given N_steps and its inclusive cumsum (total =
 * last entry), writes rays_pts [total,3], mask_outbbox [total], ray_id,
 * step_id [total] (int64). */
int pvdb_ray_sample_points(const float* rays_o, const float* rays_d, int32_t n_rays,
                           const float xyz_min[3], const float xyz_max[3], float stepdist,
                           const float* t_min, const int64_t* n_steps_cumsum, int64_t total,
                           float* rays_pts, uint8_t* mask_outbbox, int64_t* ray_id,
                           int64_t* step_id, pvdb_stream s);

/* maskcache_lookup (render_utils_kernel.cu:373-424): out[i] = world[round(xyz*scale+shift)]
 * inside the mask's shape, else 0. */
int pvdb_maskcache_lookup(const uint8_t* world, const int32_t shape[3], const float* xyz,
                          int64_t n, const float scale[3], const float shift[3], uint8_t* out,
                          pvdb_stream s);

/* ------------------------------------------------ fused training march
 * One ray per warp over ragged per-ray sample counts. Forward fuses
 * sample_pts_on_rays + mask lookup + wld2idx + DensityVDB forward + raw2alpha
 * + alpha2weight + both fast_color_thres compactions + ColorVDB forward
 * (dvgo.py:296-341). Backward recomputes transmittance from the saved per-ray
 * alpha lists (alpha2weight_backward + raw2alpha_backward) and reduces the
 * density and k0 voxel gradients with one deterministic leaf-sorted segmented
 * reduction. All buffers device, no host synchronisation.                    */

typedef struct pvdb_march_params {
  float xyz_min[3];
  float xyz_max[3];
  float near_;            /* near plane (render_kwargs['near']) */
  float far_;             /* forced to 1e9 by the reference (dvgo.py:284) */
  float stepdist;         /* stepsize * voxel_size (dvgo.py:287) */
  float act_shift;        /* density bias (dvgo.py:48) */
  float interval;         /* stepsize * voxel_size_ratio (dvgo.py:309) */
  float fast_color_thres; /* alpha and weight threshold (dvgo.py:319-335) */
  float t_stop;           /* transmittance early stop (1e-3 in the reference) */
  float bg;               /* background colour (dvgo.py:370) */
} pvdb_march_params;

/* Workspace for up to max_rays rays of at most samples_cap samples each. */
int pvdb_march_create(int32_t max_rays, int32_t samples_cap, pvdb_march* out);
int pvdb_march_destroy(pvdb_march m);

/* Leaf staging of the forward's density pass (a GB300 option, off by default;
 * no counterpart in the reference): each ray's block copies the density leaves
 * its evaluated samples interpolate from into shared memory with 1-D bulk
 * copies (up to 24 leaves of 2 KB; the rest are read from global memory) and
 * interpolates there. Results are bitwise those of the default pass. Applies
 * to forwards (and train-step captures) made after the call. */
int pvdb_march_set_leaf_staging(pvdb_march m, int32_t on);

/* Upper bound on the per-ray sample count for a bbox and step distance. */
int32_t pvdb_march_samples_cap(const float xyz_min[3], const float xyz_max[3], float stepdist);

/* Forward. rays_o/rays_d: [R,3]; mask (optional, may be NULL): dense occupancy
 * [mask_shape] used as MaskGrid (grid.py:234-243). k0 may be NULL (density only).
 * Results stay in the workspace; read them with pvdb_march_views. */
int pvdb_march_forward(pvdb_march m, pvdb_grid density, pvdb_grid k0, const float* rays_o,
                       const float* rays_d, int32_t n_rays, const pvdb_march_params* p,
                       const uint8_t* mask, const int32_t mask_shape[3], pvdb_stream s);

typedef struct pvdb_march_views_t {
  /* per ray [R] */
  float* alphainv_last;   /* transmittance after the last composited sample */
  int32_t* n_kept;        /* samples with alpha > thres before the early stop */
  int32_t* n_color;       /* of those, samples with weight > thres */
  int32_t* color_offset;  /* exclusive scan of n_color */
  /* per colour sample row [M_max] */
  float* k0;              /* [M, k0_channels] trilinear k0 features */
  float* weight;          /* [M] */
  float* alpha;           /* [M] */
  int32_t* ray_id;        /* [M] */
  int32_t* step_id;       /* [M] */
  /* device scalars */
  int32_t* totals;        /* [0] = total kept, [1] = total colour rows (M) */
  int64_t rows_capacity;  /* M_max */
} pvdb_march_views_t;

int pvdb_march_views(pvdb_march m, pvdb_march_views_t* v);

/* Host copy of the totals (synchronises the stream). */
int pvdb_march_totals(pvdb_march m, int64_t* total_kept, int64_t* total_rows, pvdb_stream s);
/* Counts of the last forward (synchronises s): kept samples, colour rows, and
 * samples marched (every ray's N_steps samples, as sample_pts_on_rays makes
 * them, up to samples_cap). No reference counterpart: the reference
 * materialises these as tensor sizes. */
int pvdb_march_stats(pvdb_march m, int64_t* kept, int64_t* rows, int64_t* evaluated,
                     pvdb_stream s);
/* Voxel counts of the last pvdb_train_step run under the stage profiler
 * (synchronises s): out[4] = {density voxels visited, density voxels updated,
 * k0 voxels visited, k0 voxels updated} by the voxel Adam (visited: the
 * active voxels of the touched leaves; updated: those with a nonzero
 * gradient). Zeros until a profiled step ran. No reference counterpart: it
 * feeds the byte model of the TV and Adam stages. */
int pvdb_march_adam_counts(pvdb_march m, int64_t* out, pvdb_stream s);

/* Backward. grad_weight [M] (per colour row), grad_last [R], grad_k0 [M, C] (may
 * be NULL when k0 is NULL or gets no gradient). Adds into density->grad and
 * k0->grad. */
int pvdb_march_backward(pvdb_march m, pvdb_grid density, pvdb_grid k0, const float* grad_weight,
                        const float* grad_last, const float* grad_k0, pvdb_stream s);

/* Deterministic per-ray composite (segment_coo sum + bg, dvgo.py:365-370):
 * rgb_marched[r] = sum_m weight[m]*rgb[m] + alphainv_last[r]*bg over rows of ray r.
 * rgb may be NULL when the forward kept no colour row (M == 0): no row is read. */
int pvdb_composite_forward(pvdb_march m, const float* rgb, float bg, float* rgb_marched,
                           int32_t n_rays, pvdb_stream s);
/* grad_rgb[m] = weight[m]*g[r]; grad_weight[m] = dot(g[r], rgb[m]);
 * grad_last[r] += bg*sum(g[r]) (added into grad_last, which the caller zeroes). */
int pvdb_composite_backward(pvdb_march m, const float* rgb, const float* grad_rgb_marched,
                            float bg, float* grad_rgb, float* grad_weight, float* grad_last,
                            int32_t n_rays, pvdb_stream s);

/* ------------------------------------------------------------- rgbnet
 * The colour MLP (dvgo.py:91-107, :354-362): input [k0 (C0), viewdir PE
 * (3+6*pe)] -> width -> width -> 3, ReLU, followed by sigmoid. Weights are FP32
 * in torch nn.Linear layout ([out,in] row-major): w0 [width, C0+3+6*pe],
 * w1 [width,width], w2 [3,width]. The PE part of layer 0 is computed once per
 * ray (renderer.cu:100-101). precision 0 = FP32 SIMT, 1 = BF16 tensor cores
 * (FP32 accumulate).                                                         */

typedef struct pvdb_mlp_weights {
  const float* w0; const float* b0;
  const float* w1; const float* b1;
  const float* w2; const float* b2;
  int32_t c0;      /* k0 channels feeding the MLP */
  int32_t pe;      /* viewbase_pe frequencies */
  int32_t width;   /* hidden width (128) */
} pvdb_mlp_weights;

/* rgb[m] = sigmoid(MLP([k0[m], PE(viewdirs[ray_id[m]])])) for rows m < totals[1]
 * of the march workspace (ray ids from the workspace). k0 [M, c0] is the
 * caller's feature rows; NULL uses the workspace's k0 rows. */
int pvdb_mlp_forward(pvdb_march m, const pvdb_mlp_weights* w, const float* k0,
                     const float* viewdirs, float* rgb, int32_t precision, pvdb_stream s);

typedef struct pvdb_mlp_grads {
  float* w0; float* b0; float* w1; float* b1; float* w2; float* b2; /* overwritten */
} pvdb_mlp_grads;

/* Given grad_rgb [M,3] (gradient w.r.t. the sigmoid output) and rgb, writes the
 * weight gradients (deterministic: fixed-order reduction of per-CTA partials)
 * and grad_k0 [M, c0]. */
int pvdb_mlp_backward(pvdb_march m, const pvdb_mlp_weights* w, const float* k0,
                      const float* viewdirs, const float* rgb, const float* grad_rgb,
                      pvdb_mlp_grads* g, float* grad_k0, int32_t precision, pvdb_stream s);

/* ------------------------------------------------------- fused train step
 * One fine-stage iteration (run.py:516-598) on device-resident rays:
 * march forward, rgbnet, composite, the reference losses (MSE, entropy of
 * alphainv_last, per-point rgb; run.py:551-575), full backward, optional TV on
 * both grids (run.py:578-584), voxel Adam on both grids (mode 1, skip zero
 * grad: configs/default.py:76), dense Adam on the rgbnet, lr decay. No host
 * synchronisation; loss written to loss_out[0] on the device.               */

typedef struct pvdb_train_config {
  pvdb_march_params march;
  float weight_main, weight_entropy_last, weight_rgbper;
  float tv_weight_density, tv_weight_k0; /* 0 disables; scaled as dvgo.py:245-251 */
  int32_t tv_dense_mode;
  float lr_decay_factor;                 /* applied after the step (run.py:592-598) */
  float rgbnet_lr, rgbnet_beta1, rgbnet_beta2, rgbnet_eps;
  int32_t precision;                     /* 0 FP32, 1 BF16 rgbnet */
  int32_t use_graph;                     /* 1: replay the step as a captured CUDA graph
                                            (captured once the same buffers, configuration
                                            and loss_out were seen twice in a row; a call
                                            with other ones runs eagerly and recaptures) */
  int32_t tv_in_place;                   /* sparse TV (tv_dense_mode 0): 0 computes the TV
                                            terms beside the gradient sums and the voxel
                                            Adam adds them to the channels with a gradient;
                                            1 adds them to the gradient in place first, as
                                            the reference does. The same values either way */
} pvdb_train_config;

typedef struct pvdb_rgbnet_state {
  float* params;      /* flat [w0,b0,w1,b1,w2,b2] FP32 master weights */
  float* grads;       /* same size */
  float* exp_avg;     /* same size */
  float* exp_avg_sq;  /* same size */
  int32_t* step;      /* host-side step counter (incremented by the call) */
  float* lr;          /* host-side lr (decayed by the call) */
  int32_t c0, pe, width;
} pvdb_rgbnet_state;

int pvdb_train_step(pvdb_march m, pvdb_opt density_opt, pvdb_opt k0_opt,
                    pvdb_rgbnet_state* net, const float* rays_o, const float* rays_d,
                    const float* viewdirs, const float* target, int32_t n_rays,
                    const pvdb_train_config* cfg, float* loss_out, pvdb_stream s);

/* ------------------------------------------------------ merged renderer
 * MGRenderer (plenvdb.h:933-1068, renderer.cu:122-424): inference over a
 * merged index grid (voxel -> row, row 0 = empty) and packed rows.          */

int pvdb_renderer_create(int32_t dcol, int32_t dpe, int32_t dhid, int32_t dout,
                         pvdb_renderer* out);
int pvdb_renderer_destroy(pvdb_renderer r);

/* load_data (plenvdb.h:959-983): index [reso] dense row ids (0 = empty; the
 * voxels with a nonzero row are the active ones), density [N], features
 * [N, dcol] (row 0 must be zeros). storage 0 = FP32 rows, 1 = BF16 features
 * with FP32 density. */
int pvdb_renderer_load_data(pvdb_renderer r, const int32_t reso[3], const int32_t* index,
                            const float* density, const float* features, int64_t n_rows,
                            int32_t storage, int32_t mem);
/* load_params (plenvdb.h:984-990): w as [in,out] row-major (run.py:98-104). */
int pvdb_renderer_load_params(pvdb_renderer r, const float* w0, const float* b0,
                              const float* w1, const float* b1, const float* w2,
                              const float* b2);
/* setScene (plenvdb.h:991-994). */
int pvdb_renderer_set_scene(pvdb_renderer r, const int32_t reso[3], const float K[9],
                            const float xyz_min[3], const float xyz_max[3]);
/* setKwargs (plenvdb.h:995-1020); far is forced to 1e9 as in the reference.
 * t_stop is the early-termination transmittance (1e-3 in the reference). */
int pvdb_renderer_set_kwargs(pvdb_renderer r, float near_, float far_, float stepdist,
                             float act_shift, float interval, float fast_color_thres,
                             float bg, int32_t inverse_y, int32_t h, int32_t w, float t_stop);
/* input_a_c2w (plenvdb.h:1022-1025): c2w [16] row-major 4x4. */
int pvdb_renderer_input_c2w(pvdb_renderer r, const float* c2w, int32_t mem, pvdb_stream s);
/* render_an_image (plenvdb.h:1027-1037) into the renderer's device image. */
int pvdb_renderer_render(pvdb_renderer r, int32_t precision, pvdb_stream s);
/* output_an_image (plenvdb.h:1038-1046): [H*W*3]. */
int pvdb_renderer_output(pvdb_renderer r, float* out, int32_t mem, pvdb_stream s);
/* Device pointer of the image [H*W*3] and the sample count of the last frame
 * (device scalar). */
int pvdb_renderer_views(pvdb_renderer r, float** image, int32_t** n_samples_total);

/* ------------------------------------------------------- grid lifecycle
 * The steps of the DVGO schedule around the training step (run.py:430-512):
 * merged-row compression for the renderer, progressive rescaling, the
 * occupancy (mask-cache) builds, near-camera masking, per-voxel view counts,
 * and the training-ray generation of the in-mask-cache sampler. Device
 * buffers only. Calls that return a count synchronise the stream.            */

/* Number of nonzero bytes of mask [n] (the N of vdb_compression.py:27-29). */
int pvdb_merge_count(const uint8_t* mask, int64_t n, int64_t* n_active, pvdb_stream s);

/* vdb_compression.py:19-59 without the file I/O: the voxels with a nonzero
 * mask byte (mask [rx*ry*rz], C order) get row ids 1..N in C order, written
 * to index [rx*ry*rz] (0 = empty); row 0 of den_rows [N+1] and col_rows
 * [(N+1)*C] is zero, row r holds the voxel's density and its C colour
 * channels (copyToArray values: the background outside allocated leaves).
 * row_dtype 0 = FP32, 1 = FP16 (the reference's mergeddata.npz). density or
 * color may be NULL (then its rows are not written). n_rows must be N+1; it
 * is checked before anything is written. Synchronises. */
int pvdb_merge_build(pvdb_grid density, pvdb_grid color, const uint8_t* mask, int32_t* index,
                     void* den_rows, void* col_rows, int64_t n_rows, int32_t row_dtype,
                     pvdb_stream s);

/* Stable compaction of up to four [n,3] float arrays by keep [n] (nonzero =
 * kept): dst[k] receives the kept rows of src[k] in order. cap is the row
 * capacity of every dst (checked before writing); *n_kept the kept count.
 * Synchronises. */
int pvdb_compact_rows(const uint8_t* keep, int64_t n, const float* const* src, float* const* dst,
                      int32_t n_arrays, int64_t cap, int64_t* n_kept, pvdb_stream s);

/* VDBGrid.scale_volume_grid (lib/grid.py:91-102): every voxel of dst's
 * allocated leaves inside its resolution gets F.interpolate(trilinear,
 * align_corners=True) of src's dense values (background outside src's
 * leaves). src and dst have the same channel count. */
int pvdb_grid_resample(pvdb_grid src, pvdb_grid dst, pvdb_stream s);

/* Occupancy (mask-cache) builds over the density grid, mask [shape] bytes:
 *  mode 0  update_occupancy_cache (lib/dvgo.py:200-210): density trilinear at
 *          the linspace(xyz_min, xyz_max, shape) points, raw2alpha, 3^3 max
 *          pool, mask &= pooled > thres (fast_color_thres); any shape;
 *  mode 1  the rebuild after scale_volume_grid (lib/dvgo.py:186-197): shape
 *          = grid resolution; raw2alpha of the voxel values, 3^3 max pool,
 *          mask = old_mask lookup at the new grid points & pooled > thres
 *          (old_mask [old_shape], NULL = all true);
 *  mode 2  MaskGrid from a checkpoint (lib/grid.py:214-221): shape = grid
 *          resolution; 3^3 max pool of the voxel values, then
 *          mask = 1 - exp(-softplus(pooled + act_shift) * interval) >= thres.
 * Values outside [0, shape) are the pool's padding (ignored). */
int pvdb_occupancy(pvdb_grid density, int32_t mode, uint8_t* mask, const int32_t shape[3],
                   const float xyz_min[3], const float xyz_max[3], float act_shift,
                   float interval, float thres, const uint8_t* old_mask,
                   const int32_t old_shape[3], pvdb_stream s);

/* maskout_near_cam_vox (lib/dvgo.py:163-175): active voxels whose grid point
 * (linspace over the resolution) lies within near_clip of any of the camera
 * centres cam_o [n_cams,3] get `value` (-100 in the reference). */
int pvdb_grid_maskout_near_cams(pvdb_grid g, const float* cam_o, int32_t n_cams,
                                const float xyz_min[3], const float xyz_max[3], float near_clip,
                                float value, pvdb_stream s);

/* voxel_count_views for one view (lib/dvgo.py:212-243): every ray takes
 * n_samples points t_min + stepdist*k/|d| (stepdist = stepsize*voxel_size),
 * each point adds its trilinear weights to the voxels it touches (zero
 * padding), and count [reso] += (sum > 1). acc [reso] is uint64 scratch that
 * must be zero on entry and is zero again on return (32.32 fixed-point sums:
 * exact and independent of the order of the atomics). */
int pvdb_count_views(const float* rays_o, const float* rays_d, int64_t n_rays,
                     const int32_t reso[3], const float xyz_min[3], const float xyz_max[3],
                     float near_, float stepdist, int32_t n_samples, uint64_t* acc, float* count,
                     pvdb_stream s);

/* get_rays_of_a_view (lib/dvgo.py:471-521): rays_o, rays_d, viewdirs [H*W,3]
 * of a pinhole view, pixels in row-major (h, w) order. K [9] row-major (the
 * reference's float64 intrinsics), c2w [16] row-major 4x4 (host). mode 0 =
 * 'center', 1 = 'lefttop', 2 = 'random' with jitter [2][H*W] (device) holding
 * the uniform offsets of i then j before the flips. ndc applies ndc_rays with
 * near 1 and focal K[0] to rays_o/rays_d (viewdirs stay those of the pinhole
 * rays). */
int pvdb_get_rays(int32_t H, int32_t W, const double K[9], const float c2w[16], int32_t ndc,
                  int32_t inverse_y, int32_t flip_x, int32_t flip_y, int32_t mode,
                  const float* jitter, float* rays_o, float* rays_d, float* viewdirs,
                  pvdb_stream s);

/* hit_coarse_geo (lib/dvgo.py:258-270): hit[r] = 1 when a sample of
 * sample_pts_on_rays (far = 1e9) inside the bbox lands in a nonzero voxel of
 * the mask cache mask [shape] (nearest lookup, MaskGrid scale/shift). */
int pvdb_rays_hit_mask(const float* rays_o, const float* rays_d, int64_t n,
                       const float xyz_min[3], const float xyz_max[3], float near_,
                       float stepdist, const uint8_t* mask, const int32_t shape[3], uint8_t* hit,
                       pvdb_stream s);

#ifdef __cplusplus
}
#endif
#endif /* PVDB_H */
