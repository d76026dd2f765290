/*
 * sonar_render.h -- C ABI of the GB300 discrete Kirchhoff library
 * (libsonar_gb300.so, also shipped as build/libcuda_project.so).
 *
 * The first block keeps the reference's python_interface symbols and
 * signatures so existing ctypes callers (run_scripts/modules/api.py:4-111)
 * load this library unchanged.  Each declaration cites the reference entry
 * point it replaces (src/python_interface.cpp).  Like the reference they
 * return void; unlike the reference they never throw across the boundary:
 * an error is recorded (sonar_status / sonar_last_error) and the call, and
 * every later projection until TearDownCuda, does nothing.
 *
 * The second block is additive: status, headless surface-pressure read-back
 * (the reference only exposes surfaces through GL textures,
 * src/FacetCuda.cu:74-85), fragment layout, statistics, options and the
 * interaction mask (test/diagnostic use).
 *
 * Pointers are plain host pointers; sizes are element counts.  The library
 * owns all device memory (returned to its memory pool by TearDownCuda; see
 * the options "memory_cache_mb" and "release_memory").  Calls are synchronous and
 * not thread-safe, as in the reference (one process-global model,
 * src/python_interface.cpp:11).
 */
#ifndef SONAR_RENDER_H
#define SONAR_RENDER_H

#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Complex pressure, two doubles (src/dcomplex.h:12-15). */
typedef struct DCOMPLEX {
    double r, i;
} dcomplex;

/* ---- reference entry points (src/python_interface.cpp) ------------------ */

/* :21-24 -- k = (float)(2*pi*f) / cp, attenuation is the imaginary part of k
 * in Np/m (src/Model.cpp:44-54); density is stored and unused. */
void set_initial_conditions(float cp, float frequency, float attenuation, float density);

/* :26-41 -- num_vertices counts TRIANGLES (9 floats each: v1 v2 v3);
 * objectType 0 target, 1 source (stored, unused), 2 field surface;
 * resolution is the fragment side delta in metres. */
void load_geometry(float *v1, int num_vertices, int objectType, float resolution);

/* :43-50 -- xyz triples; field point pressures start at 0 and accumulate. */
void load_field_points(float *v1, int num_feild_points);

/* :52-59 -- xyz triples; every source has pressure 1 + 0i (src/Model.cpp:16-19). */
void load_source_points(float *v1, int num_source_points);

/* :61-65 -- fragment every target and field facet (src/Facet.cpp:111-339),
 * build the occluder BVH over all target triangles (replaces the OptiX GAS,
 * src/OptiX.cpp:264-350) and upload the scene.  No projection runs here. */
void render_cuda(void);

/* :67-70 -- source points -> every target object (and every field object when
 * projectFieldObjects), src/ModelCuda.cpp:242-278, src/OptiX.cu:35-110. */
void ProjectSrcPointsToObjects(bool projectFieldObjects);

/* :72-75 -- target objects -> field objects (FACET_NO_RESP),
 * src/ModelCuda.cpp:280-301, src/OptiX.cu:192-406. */
void ProjectTargetToFieldObjects(void);

/* :77-80 -- target objects -> field points, src/ModelCuda.cpp:302-321,
 * src/OptiX.cu:112-190. */
void ProjectTargetToFieldPoints(void);

/* :82-85 -- number_reflections fragment -> fragment bounces per target object
 * (FACET_SELF with reciprocity), src/ModelCuda.cpp:323-356. */
void ProjectTargetToTargetObjects(int number_reflections);

/* :87-90 -- copy the field point pressures (load order).  The reference copies
 * every loaded point whatever NumPoints says (src/ModelCuda.cpp:203-208); this
 * copies min(NumPoints, loaded) and records an error when NumPoints is short. */
void GetFieldPointPressures(dcomplex *field_points_pressure, int NumPoints);

/* :92-96 -- the picture the reference draws through EGL/GL (every facet of the
 * target and field objects textured with its pressure colour map, camera
 * glm::perspective(45 deg, width/height, 0.1, 10000) * glm::lookAt(eye =
 * viewSettings[0..2], centre = [3..5], up = [6..8]), ModelGl.cpp:98-106,
 * 222-341), rasterised by CUDA kernels instead (no graphics stack is needed)
 * and written to `filename` as an RGB PNG, top row first.  Triangles with a
 * vertex behind the near plane are not drawn. */
void RenderOpenGL(int width, int height, char *filename, float viewSettings[9]);

/* :98-101 -- free all device memory, drop target/field objects and points
 * (src/Model.cpp:115-129, src/ModelCuda.cpp:124-181) and clear the error. */
void TearDownCuda(void);

/* :103-107 -- store the dB window and phase flags used by surface colouring. */
void SoundVisualisationInit(float maxDbValue, float minDbValue, bool renderPhaseTarget, bool renderPhaseField);

/* ---- additive entry points ---------------------------------------------- */

/* 0 when no error is pending, else a negative code. */
int sonar_status(void);
/* Message of the pending error ("" when none). */
const char *sonar_last_error(void);
/* Clear a pending error (loads and projections run again). */
void sonar_clear_error(void);

/* Number of loaded objects of a type (0 target, 1 source, 2 field). */
int sonar_get_object_count(int objectType);
/* Cells of an object after render_cuda: sum over facets of numXpnts*numYpnts. */
long long sonar_get_object_cells(int objectType, int objIdx);
/* Total pressure P of every cell of a target or field object: facet-major,
 * each facet row-major y*numXpnts + x (src/OptiX.cu:49).  n is the capacity
 * in dcomplex; returns the number written or a negative code. */
int sonar_get_object_pressures(int objectType, int objIdx, dcomplex *out, long long n);
/* Fragment layout of an object: 3 ints per facet (numXpnts, numYpnts,
 * numXpntsNegative, src/Facet.cpp:124-127) and the FP32 cell areas in the
 * same order as the pressures.  Returns the number of facets or < 0. */
int sonar_get_fragment_layout(int objectType, int objIdx, int *nx_ny_neg, int nfacets_cap, float *areas,
                              long long ncells_cap);
/* Surface colours of a target or field object: 4 floats (RGBA in [0, 1]) per
 * cell in the pressure layout, the texel values the reference writes into its
 * GL textures (MakeSurface, src/FacetCuda.cu:43-72) with the dB window and
 * phase flags of SoundVisualisationInit.  Returns the number of cells written
 * or < 0. */
int sonar_get_surface_colours(int objectType, int objIdx, float *rgba, long long ncells);
/* The picture of RenderOpenGL into a caller buffer: height rows of width x 3
 * bytes (RGB), top row first.  Returns 0 or a negative code. */
int sonar_render_image(int width, int height, const float *viewSettings, unsigned char *rgb);
/* JSON statistics of the last projection calls (pairs, kernel ms, grazing). */
int sonar_get_stats(char *json, int cap);
/* Options: "split" (source splits of the sum kernels, 0 = automatic),
 * "f2f_symmetric" (1, default: bounce sums evaluate each unordered pair once
 * and feed both directions, as the reference's reciprocity does; 0: every
 * ordered pair separately),
 * "verbose" (0/1), "reset_stats", "reset_pressures" (zero every surface and
 * field-point pressure), "drop_masks" (rebuild the cached interaction masks,
 * in place, at their next use), "free_masks" (free them), "class_stats"
 * (count the mask's block classes), "mask_classify" (1, default: bounce
 * masks classify their blocks one warp per block and build per-pair bits
 * only for the blocks that need them; 0: every block in the pair kernel),
 * "mask_gate_proj" (1, default: the pair kernel decides gates from per-point
 * projections where that is certain; 0: every pair's gates evaluated).
 * "cross_objects" (0, default: bounces stay within each target, as in the
 * reference's ProjectTargetToTargetObjects; 1: every bounce also carries
 * the terms between every pair of targets -- the reference's FACET_RESP
 * projection, src/OptiX.cu:192-406, :427-429, which its host never calls --
 * forward into the higher-index object, reciprocal into the lower, all
 * from the bounce's inputs).
 * "aca_variant" (cross-approximation kernel shape, 0-2; bit-identical).
 * "tile_align" (1, default: each facet's full 16 x 16-cell patches start on
 * 256-fragment tile boundaries and its edge cells -- readout centroid on or
 * outside the triangle -- come last; 0: plain patch order; the order is
 * internal, outputs are the same up to FP32 summation order; read by
 * render_cuda).
 * "ip_transpose" (0, default: an interpolation tile's first axis is the
 * fragment grid's x axis; 1: a tile whose box is taller than wide takes the
 * grid's y axis first, so that strips of partial patches along a slanted
 * facet edge fit the 32 x 16-cell box -- more blocks interpolated, no faster
 * on the 60 kHz trihedral).
 * "overlap_streams" (1, default: a compressed bounce runs its low-rank apply
 * on a second stream beside the dense remainder, joined before the
 * finalize; 0: one stream; the same results either way).
 * Device memory: every buffer comes from a stream-ordered pool kept for the
 * process; "memory_cache_mb" (32768, default: unused pool memory kept at a
 * synchronisation point, in MiB; 0 gives it all back there; negative: -6),
 * "release_memory" (wait for the device and give the pool's unused memory
 * back now).  The statistics report "pool_reserved_bytes" (memory the pool
 * has mapped) and "render_host_ms" (host time of the last render_cuda:
 * setup, fragments, uploads, occluders, points).
 * Low-rank bounce blocks (no counterpart in the reference, which evaluates
 * every pair): "compress" (0/1), "compress_tol" (cross-approximation stopping
 * tolerance, 1e-4), "compress_judge" (largest accepted relative RMS error of
 * a block on its sampled exact entries, 3e-4), "compress_rmax" (rank cap,
 * 32, at most 64), "compress_select" (which blocks are approximated: 0 those
 * whose every pair interacts and whose tiles are farther apart than
 * "compress_eta" (1.0) times the sum of their radii; 1 every interacting
 * block; 2 the blocks the admissibility network proposes), "compress_rcut"
 * (the network proposes blocks with predicted rank below this, 32).
 * Returns 0, or < 0 for an unknown key or a failed action. */
int sonar_set_option(const char *key, double value);
/* The library's CUDA stream (a cudaStream_t; NULL before render_cuda), for
 * callers that time or order work against it. */
void *sonar_get_stream(void);
/* Throughput probe of the current device for roofline denominators:
 * which = 0 FP32 fused multiply-add rate in FLOP/s, which = 1 MUFU (sine)
 * rate in op/s.  Runs for a few milliseconds; < 0 on failure. */
double sonar_measure_peak(int which);
/* Interaction mask of one hop, for diagnostics: one byte per (destination,
 * source) pair, destination-major, 1 when the pair passes the area, cosine
 * and visibility gates.  hop 0 sources -> cells of object dstIdx of type
 * srcIdx (0 target, 2 field); hop 1 active cells of target srcIdx -> field
 * points; hop 2 active cells of target srcIdx -> themselves; hop 3 active
 * cells of target srcIdx -> active cells of field object dstIdx; hop 4
 * (FACET_RESP) active cells of target srcIdx -> active cells of target
 * dstIdx != srcIdx.  Returns the number of bytes (ndst*nsrc), or < 0.  The
 * mask is built if needed. */
long long sonar_get_mask(int hop, int srcIdx, int dstIdx, unsigned char *out, long long cap);
/* The same for the destination rows rows[0..nrows) only (indices in the
 * order sonar_get_mask uses), row q at out[q * nsrc]: for masks too large to
 * export whole.  Returns nrows * nsrc, or < 0. */
long long sonar_get_mask_rows(int hop, int srcIdx, int dstIdx, const int *rows, int nrows, unsigned char *out,
                              long long cap);

/* Audit of the last compressed bounce's accepted blocks (no counterpart in
 * the reference): for up to nsample of them, chosen by seed, the relative RMS
 * error of the low-rank factors over every entry of the 256 x 256 block
 * (full_err) beside the error the judge measured on its 512 sampled entries
 * (judged_err).  Needs a compressed bounce of a target without attenuation
 * and a build with FP32 factors.  Returns the number of blocks audited, or
 * < 0 (sonar_last_error). */
int sonar_audit_compression(int nsample, unsigned seed, float *full_err, float *judged_err, int cap);

/* Host only (no GPU needed): frame and clipped area grid of one triangle
 * (src/Facet.cpp:6-339).  nx_ny_neg gets numXpnts, numYpnts,
 * numXpntsNegative; frame17 gets normal(3) base point(3) xAxis(3) yAxis(3)
 * BaseLength Height BaseLengthNeg BaseLengthPos Area; areas (row-major
 * y*numXpnts + x) is written when cap holds every cell.  Returns the cell
 * count, or < 0 for invalid arguments. */
long long sonar_fragment_triangle(const float *tri9, float delta, int *nx_ny_neg, float *frame17, float *areas,
                                  long long cap);
/* Host only (no GPU needed), no counterpart in the reference: the order in
 * which render_cuda stores one triangle's active fragments when its first
 * active fragment has index start in the object (option "tile_align", on by
 * default): xy gets (x, y) grid cells, 2 ints per active fragment, when cap
 * holds them all.  Full 16 x 16-cell patches start on 256-fragment tile
 * boundaries; partial patches follow the triangle's boundary; cells whose
 * readout centroid lies on or outside the triangle come last.  Returns the
 * number of active fragments, or < 0 for invalid arguments. */
long long sonar_tile_order(const float *tri9, float delta, long long start, int *xy, long long cap);

/* Admissibility network for the low-rank bounce blocks (no counterpart in the
 * reference): a perceptron 8 -> w -> w -> w -> 1 with ReLU, hidden width w =
 * 64 (default) or 128, trained in FP32 and run by the library's own CUDA
 * kernels (width 64: FP32 inference on the CUDA cores; width 128: FP16
 * hidden layers on the tensor cores with FP32 accumulation, input and
 * output layers FP32).  Input: 8 descriptors
 * of a block (log2(1 + separation / lambda), log2(1 + radius / lambda) of the
 * source and destination tiles, cosines of both mean normals with the
 * separation direction and with each other, (r_I + r_J) / separation capped
 * at 4, fraction of interacting pairs); output: predicted log2(1 + rank).
 * Parameters: per layer the weights (out x in, row-major) then the biases.
 * Every call returns 0 or a negative code (sonar_last_error). */
int sonar_mlp_param_count(void);
/* Hidden width 64 or 128; drops the parameters (initialise or load again). */
int sonar_mlp_set_width(int width);
int sonar_mlp_width(void);
int sonar_mlp_init(unsigned seed); /* He-uniform weights, zero biases */
int sonar_mlp_set_params(const float *params, long long n);
int sonar_mlp_get_params(float *params, long long n);
/* Mean squared error of (X: n x 8, y: n) and its gradient (param_count floats). */
int sonar_mlp_grad(const float *X, const float *y, int n, float *grad, float *loss);
/* Adam (beta 0.9, 0.999, eps 1e-8) over seeded shuffled mini-batches; loss
 * gets the mean squared error of the last epoch. */
int sonar_mlp_train(const float *X, const float *y, int n, int epochs, int batch, float lr, unsigned seed,
                    float *loss);
int sonar_mlp_predict(const float *X, int n, float *out);
/* Descriptors (n x 8) and rank labels (n; log2(1 + rank), or log2(1 + 2 cap)
 * for blocks the judge rejected) of the blocks approximated by the last
 * compressed bounce.  Returns n; copies when cap >= n. */
long long sonar_get_block_samples(float *X, float *y, long long cap);

/* Many sources, receivers, frequencies and scenes at once (the reference's
 * run scripts loop over these on the host, one render per source and
 * frequency: load_source_points / set_initial_conditions /
 * ProjectSrcPointsToObjects / ProjectTargetToFieldPoints /
 * GetFieldPointPressures, src/python_interface.cpp:21-90).  For every scene s
 * (triangles tris[9*scene_tri_off[s] .. 9*scene_tri_off[s+1]), all of them
 * target objects), frequency f (fragment size cp / f / per_wavelength, k as
 * set_initial_conditions computes it), receiver p and source q, out holds the
 * field-point pressure at p when source q alone radiates with unit pressure:
 * the source hop onto every fragment cell then the readout of the target
 * fragments, both shadowed like the reference's.  Layout: out[((s*nfreq + f)
 * * nrx + p) * nsrc + q] as 2 doubles (re, im).  At most 64 sources and 64
 * receivers.
 *
 * sonar_batch_plan fragments every (scene, frequency) item on the host,
 * uploads it, times the candidate tile shapes and captures the run as a CUDA
 * graph; it returns a plan id (> 0) or a negative code.  sonar_batch_run
 * replays the graph (interaction masks, one persistent tensor-core launch,
 * reduction) and copies the result into out (NULL: leave it on the device).
 * sonar_batch_stats writes JSON (items, fragments, credited pairs, kernel
 * times of the last run, the tuning chosen and every candidate's time) and
 * returns its length.  sonar_batch_stream gives the plan's cudaStream_t.
 * sonar_run_batch = plan, run, free.  Plans are independent of the
 * single-scene model above.  Return 0 or a negative code (sonar_last_error). */
long long sonar_batch_plan(const float *tris, const int *scene_tri_off, int nscenes, const float *src_xyz, int nsrc,
                           const float *rx_xyz, int nrx, const float *freqs, int nfreq, float cp, float attenuation,
                           float per_wavelength);
int sonar_batch_run(long long plan, double *out);
int sonar_batch_stats(long long plan, char *json, int cap);
/* New source and receiver positions for the next sonar_batch_run of a plan
 * (the same counts as planned), as a sequence of pings moves them: the
 * geometry, its fragments and the tuning are kept; the run recomputes the
 * visibility words.  Returns 0 or a negative code. */
int sonar_batch_set_points(long long plan, const float *src_xyz, int nsrc, const float *rx_xyz, int nrx);
/* Replace the tuned tile shape of a plan (diagnostics and tests): fragments
 * per operand stage 16, 32 or 64 and persistent CTAs per SM (as many as
 * shared memory holds, at most 4); the run graph is captured again.  Returns
 * 0 or a negative code. */
int sonar_batch_set_shape(long long plan, int fragments_per_stage, int ctas_per_sm);
/* Centroid-relative phase for a plan (on != 0), no counterpart in the
 * reference: the reference forms each distance from absolute FP32 positions
 * (src/OptiX.cu:45-57, :150-153), which at a 30 m range rounds the phase by
 * about 2e-4 rad at 40 kHz.  With it on, every point is taken relative to its
 * scene's box centre c in FP64 on the host (D = point - c, R = |D|, k R
 * reduced to turns) and the kernel forms the phase distance as
 * R + (|o|^2 - 2 o.D) / (r + R) with o = fragment - c.  Off by default
 * (parity with the reference's rounding); the run graph is captured again.
 * Returns 0 or a negative code. */
int sonar_batch_set_relative(long long plan, int on);
int sonar_batch_stream(long long plan, void **stream);
int sonar_batch_free(long long plan);
int sonar_run_batch(const float *tris, const int *scene_tri_off, int nscenes, const float *src_xyz, int nsrc,
                    const float *rx_xyz, int nrx, const float *freqs, int nfreq, float cp, float attenuation,
                    float per_wavelength, double *out);

/* Fragment -> field-point readout that allocates no memory.  No counterpart in
 * the reference: it exists for callers that cannot call cudaMalloc while they
 * run (a host framework that owns all device memory through its own pool, a
 * real-time host that allocates only at start-up, code that must avoid the
 * synchronisation an allocation can cause).
 *
 * Computes, for every field point j, out[j] += sum over fragments i with
 * area > 1e-6 and cos_scat >= 1e-6 of area_i cos_scat P_i G(r) -- the
 * FIELD_POINTS sum of ProjectTargetToFieldPoints -- without shadowing (no
 * occlusion test), on caller-owned DEVICE buffers:
 *   frag_pos       n_frag x 4 floats: centroid x, y, z and area
 *   frag_normal    n_frag x 4 floats: unit normal x, y, z (4th unused)
 *   frag_pressure  n_frag x 2 doubles: complex pressure
 *   points         n_points x 4 floats: field point x, y, z (4th unused)
 *   out            n_points x 2 doubles: complex pressure, accumulated (+=)
 * k_re, k_im: the wave number as set_initial_conditions computes it
 * ((float)(2 pi f) / c and the attenuation).  The work is queued on `stream`
 * (a cudaStream_t, NULL for the default stream); the call does not wait.
 *
 * Every buffer must start on a 16-byte boundary (the kernels read them as
 * float4 / double2 vectors): a caller's sub-allocation or slice at another
 * offset is refused with SONAR_NOALLOC_EINVAL.  The cosine gate is decided
 * with the reference's FP32 rounding, as in the library's own readout.
 *
 * Its only working memory is a fixed 8 MiB device array inside this library
 * (held by every GPU that loads it, until the process exits), so n_points is
 * limited to SONAR_NOALLOC_MAX_POINTS.  The array's address is looked up on
 * the first call made in each CUDA context; make that first call before any
 * stream capture begins.  A context destroyed and re-created (cudaDeviceReset)
 * invalidates the cached address; the next call looks it up again, so that
 * call too must come before any capture.  All calls share the array: calls
 * whose work overlaps on the GPU (e.g. on two streams at once) race and give
 * wrong results.
 * Returns 0, SONAR_NOALLOC_EINVAL (bad size, null or misaligned pointer),
 * SONAR_NOALLOC_ETOOBIG (n_points above the maximum) or SONAR_NOALLOC_ECUDA
 * (device lookup or launch failed, or a CUDA error from the caller's own
 * work was already pending -- it is left pending; a line goes to stderr). */
#define SONAR_NOALLOC_MAX_POINTS 524288
#define SONAR_NOALLOC_EINVAL (-1)
#define SONAR_NOALLOC_ETOOBIG (-2)
#define SONAR_NOALLOC_ECUDA (-3)
int sonar_readout_noalloc(const float *frag_pos, const float *frag_normal, const double *frag_pressure, int n_frag,
                          const float *points, int n_points, float k_re, float k_im, double *out, void *stream);

#ifdef __cplusplus
}
#endif
#endif
