/*
 * fastpli_gb300 — C ABI of the GB300 (sm_103a) forward model of 3D-PLI.
 *
 * Drop-in for the two pybind11 classes fastpli's `Simpli` binds:
 *   _Generator  (src/simulation/bindings/generator_module.cpp:23-140)
 *   _Simulator  (src/simulation/bindings/simulator_module.cpp:18-157)
 * Every entry point takes plain pointers and sizes; streams are passed as
 * `void *` holding a cudaStream_t (NULL = legacy default stream).  Calls
 * return 0 on success or a negative FPGB_E* code; fpgb_last_error() then
 * holds the message (thread-local).  Argument errors the reference raises as
 * std::invalid_argument / ValueError, and the input checks it answers with
 * exit(EXIT_FAILURE) (src/simulation/simulator.cpp:62-69,131-176), are both
 * reported as FPGB_EINVAL here — nothing in this library exits the process.
 *
 * Units and layouts are the reference's: lengths in µm, wavelength in nm,
 * angles in rad; label [X][Y][Z] int32 and vector [X][Y][Z][3] float32,
 * z fastest; images [X][Y][n_rho] float64.
 */
#ifndef FASTPLI_GB300_H_
#define FASTPLI_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FPGB_OK 0
#define FPGB_EINVAL (-1)   /* invalid argument / inconsistent input */
#define FPGB_ECUDA (-2)    /* CUDA runtime error */
#define FPGB_ENOMEM (-3)   /* allocation failed / workspace too small */
#define FPGB_ETIMEOUT (-4) /* a bounded device wait gave up */

/* Counters of the reference's Python UserWarnings (PyErr_WarnEx sites). */
typedef struct fpgb_warnings {
   int64_t overlap;        /* "objects overlap" generator.cpp:357 */
   int64_t single_point;   /* "fiber object with only single point" :215 */
   int64_t zero_axis;      /* "optical_axis is 0 for tissue > 0" simulator.cpp:294 */
   int64_t not_normalized; /* "optical_axis not normalized" simulator.cpp:300 */
   int64_t empty_light;    /* "light_positions is empty" simulator.cpp:715 */
   int64_t layer_overflow; /* voxels whose layer quotient lies beyond the
                              outermost layer (generator.cpp:345-366 reads past
                              its layer table there; here: zero vector) */
} fpgb_warnings;

/* Volume of _Generator.set_volume (generator_module.cpp:29-35,
 * generator.cpp:45-124). */
typedef struct fpgb_volume {
   int64_t dim[3];
   double origin[3];
   double voxel_size;
} fpgb_volume;

/* Fiber bundles of _Generator.set_fiber_bundles (generator_module.cpp:37-66)
 * flattened: fiber f owns points [fiber_point_off[f], fiber_point_off[f+1]),
 * bundle b owns fibers [bundle_fiber_off[b], bundle_fiber_off[b+1]) and
 * layers [bundle_layer_off[b], bundle_layer_off[b+1]).  Host memory. */
typedef struct fpgb_fibers {
   int64_t n_bundles;
   const int64_t *bundle_fiber_off; /* [n_bundles + 1] */
   const int64_t *fiber_point_off;  /* [n_fibers + 1] */
   const double *points;            /* [n_points][4] = x, y, z, radius */
   const int64_t *bundle_layer_off; /* [n_bundles + 1] */
   const double *layer_scale;       /* [n_layers] */
   const double *layer_dn;
   const double *layer_mu;
   const char *layer_model; /* 'b' background, 'p' parallel, 'r' radial */
} fpgb_fibers;

/* _Simulator.set_pli_setup (simulator_module.cpp:23-54, setup.hpp:47-82). */
typedef struct fpgb_setup {
   double step_size;       /* in voxels */
   double light_intensity; /* a.u. */
   double voxel_size;      /* µm */
   double wavelength;      /* nm */
   double tissue_refrection;
   int32_t interpolate; /* 0 = NN, 1 = Lerp, 2 = Slerp */
   int32_t untilt_sensor_view;
   int32_t flip_z;
   int32_t n_rho;
   const double *filter_rotations; /* [n_rho], host memory, rad */
} fpgb_setup;

const char *fpgb_last_error(void);
const char *fpgb_version(void);

/* ----------------------------------------------------------------------------
 * Voxelizer.  Replaces _Generator.run_generation
 * (generator_module.cpp:99-134 -> PliGenerator::RunTissueGeneration,
 * generator.cpp:163-261).  n_props = 1 + n_bundles * max_layer rows of
 * (dn, mu) (generator.cpp:496-526); row 0 is (0, 0).
 * -------------------------------------------------------------------------- */

/* Host buffers in and out (copies inside): label [X*Y*Z], vector
 * [X*Y*Z*3] (unused when only_label), props [props_cap][2]. */
int fpgb_generate_tissue(const fpgb_volume *vol, const fpgb_fibers *fibers,
                         int only_label, int32_t *label, float *vector,
                         double *props, int64_t props_cap, int64_t *n_props,
                         fpgb_warnings *warnings);

/* Device-resident variant.  d_label / d_vector are device buffers of the
 * full volume; d_workspace (>= fpgb_generate_workspace_size bytes, 256-byte
 * aligned) holds the segment and layer tables and the segment lists of the
 * voxel bricks (the per-voxel winner keys stay in shared memory), or NULL to
 * use the library's own cached device pool.  props/n_props/warnings are host memory;
 * warnings != NULL synchronises the stream. */
size_t fpgb_generate_workspace_size(const fpgb_volume *vol,
                                    const fpgb_fibers *fibers);
int fpgb_generate_tissue_device(const fpgb_volume *vol,
                                const fpgb_fibers *fibers, int only_label,
                                int32_t *d_label, float *d_vector,
                                double *props, int64_t props_cap,
                                int64_t *n_props, void *d_workspace,
                                size_t workspace_bytes, fpgb_warnings *warnings,
                                void *stream);

/* Voxelizer that allocates no device memory.  No counterpart in the
 * reference (whose voxelizer runs on the host).  For callers that cannot call
 * cudaMalloc (device memory owned by another allocator, or code that must not
 * issue allocation calls): same inputs, outputs and results as
 * fpgb_generate_tissue_device, but the scratch (segment and layer tables,
 * segment lists of the 8x8x32-voxel bricks) lives in a fixed 64 MiB
 * __device__ array of this library that every GPU loading it holds until
 * exit.  Problems needing more scratch (288 bytes per fiber segment plus 4
 * per segment-brick overlap and 8 per brick: about 220,000 short segments) are
 * rejected with FPGB_EINVAL before any device work.  The first call on a device resolves the array's address with that
 * device current; make it before any stream capture.  All calls on a device
 * share the array: calls whose device work overlaps race and must be
 * serialised. */
int fpgb_generate_tissue_noalloc(const fpgb_volume *vol,
                                 const fpgb_fibers *fibers, int only_label,
                                 int32_t *d_label, float *d_vector,
                                 double *props, int64_t props_cap,
                                 int64_t *n_props, fpgb_warnings *warnings,
                                 void *stream);

/* ----------------------------------------------------------------------------
 * Ray march.  Replaces _Simulator.run_simulation
 * (simulator_module.cpp:61-93 -> PliSimulator::RunSimulation,
 * simulator.cpp:182-411).
 * -------------------------------------------------------------------------- */

/* Host buffers in and out: label [X*Y*Z], vector [X*Y*Z*3], props
 * [n_props][2] (dn, mu) -> image [X*Y*n_rho] float64. */
int fpgb_run_simulation(const fpgb_setup *setup, const int64_t *dim,
                        const int32_t *label, const float *vector,
                        const double *props, int64_t n_props, double theta,
                        double phi, double *image, fpgb_warnings *warnings);

/* Device-resident variant: d_label, d_vector, d_image on the device; props
 * on the host (a small table, copied into the launch).  Label range checks
 * (simulator.cpp:149-167) run on the device.  warnings != NULL synchronises;
 * with NULL the call is fully asynchronous and range errors are reported by
 * the next synchronising call on that stream. */
int fpgb_run_simulation_device(const fpgb_setup *setup, const int64_t *dim,
                               const int32_t *d_label, const float *d_vector,
                               const double *props, int64_t n_props,
                               double theta, double phi, double *d_image,
                               fpgb_warnings *warnings, void *stream);

/* Same march, with the epa modalities of fastpli.analysis.epa.epa
 * (src/fastpli/analysis/epa.py:9-45) fused into the epilogue: d_trans,
 * d_dir, d_ret are [X*Y] float64 (any may be NULL). */
int fpgb_run_simulation_epa_device(const fpgb_setup *setup, const int64_t *dim,
                                   const int32_t *d_label,
                                   const float *d_vector, const double *props,
                                   int64_t n_props, double theta, double phi,
                                   double *d_image, double *d_trans,
                                   double *d_dir, double *d_ret,
                                   fpgb_warnings *warnings, void *stream);

/* Several tilts of one device-resident volume: the same march as
 * fpgb_run_simulation_epa_device for each (theta[k], phi[k]) into
 * d_images[k] (and d_trans[k], d_dir[k], d_ret[k] when those arrays are
 * given; any entry may be NULL), with the tilts spread over the library's
 * own streams so that one tilt's last rays share the GPU with the next
 * tilt's first, joined back to `stream`.  Replaces the per-tilt loop of
 * run_simulation calls in Simpli.run_simulation_pipeline
 * (src/fastpli/simulation/simpli.py:337-345).  warnings, when not NULL,
 * has n_tilts entries and makes the call synchronise; with NULL it is
 * asynchronous like fpgb_run_simulation_device. */
int fpgb_run_simulations_device(const fpgb_setup *setup, const int64_t *dim,
                                const int32_t *d_label, const float *d_vector,
                                const double *props, int64_t n_props,
                                int64_t n_tilts, const double *theta,
                                const double *phi, double *const *d_images,
                                double *const *d_trans, double *const *d_dir,
                                double *const *d_ret, fpgb_warnings *warnings,
                                void *stream);

/* Number of ray-voxel steps one run_simulation call marches: X*Y rays times
 * the steps each takes (simulator.cpp:259-261), computed on the host. */
int64_t fpgb_count_steps(const fpgb_setup *setup, const int64_t *dim,
                         double theta, double phi);

/* ----------------------------------------------------------------------------
 * Optic stage after the march.  Replaces fastpli.simulation.optic
 * (src/fastpli/simulation/optic.py) as used by Simpli.apply_optic_resample /
 * apply_optic (src/fastpli/simulation/__simpli.py:462-552).
 * ------------------------------------------------------------------------- */

/* Output size of resample (optic.py:100-101): int(round(X * scale)),
 * int(round(Y * scale)), halves rounded to even. */
int fpgb_optic_resample_size(int64_t X, int64_t Y, double scale, int64_t *out_dim);

/* optic.filter_resample (optic.py:169-187) for every polarizer angle of an
 * image stack [X, Y, n_rho] (the march's layout), into [SX, SY, n_rho]:
 * Gaussian blur of width sigma / scale with scipy.ndimage.gaussian_filter
 * semantics (axis 0 then 1, mode 'reflect', truncate 4.0, FP64; sigma == 0
 * skips it), then the block-average resample of optic.py:85-120.  Device
 * buffers; stream-ordered, no synchronisation. */
int fpgb_optic_filter_resample_device(const double *d_image, int64_t X, int64_t Y,
                                      int64_t n_rho, double sigma, double scale,
                                      double *d_out, void *stream);
/* Same with host buffers (synchronous). */
int fpgb_optic_filter_resample(const double *image, int64_t X, int64_t Y, int64_t n_rho,
                               double sigma, double scale, double *out);

/* The negative-binomial CCD noise of the reference's pipelines
 * (noise_model = lambda x: np.random.negative_binomial(x / (gain - 1),
 * 1 / gain), tests/simulation/simpli_test.py:276-277): per pixel a Poisson
 * draw of a Gamma(x / (gain - 1), scale gain - 1) rate, mean x, variance
 * gain * x.  Pixel e's draw depends only on (seed, offset + e).  Pixels with
 * x <= 0 or non-finite x are copied and counted in *n_invalid (numpy refuses
 * n <= 0); when n_invalid is non-null the call synchronises to fill it.
 * Device buffers. */
int fpgb_optic_noise_device(const double *d_in, int64_t n, double gain, uint64_t seed,
                            uint64_t offset, double *d_out, int64_t *n_invalid, void *stream);

/* epa (src/fastpli/analysis/epa.py:9-45) of an image stack [n_pix, n_rho]
 * (n_rho <= 64) in FP64: transmittance, direction, retardation maps.
 * Device buffers; stream-ordered. */
int fpgb_epa_device(const double *d_image, int64_t n_pix, int64_t n_rho, double *d_t,
                    double *d_d, double *d_r, void *stream);

/* ROFL tilt analysis (src/fastpli/analysis/rofl.py:16-63 with
 * _ROFL_with_jacobi.py, as Simpli.apply_rofl applies it per pixel,
 * __simpli.py:623-705) of a 5-tilt series d_data [5, n_pix, n_rot] (tilts
 * (0,0), (tau,0), (tau,90), (tau,180), (tau,270) degrees; 4 <= n_rot <= 32),
 * FP64, one thread per pixel.  d_out [n_pix, 8] receives direction,
 * inclination, t_rel, their standard deviations, chi^2 and MINPACK's
 * evaluation count (the reference's niter).  The fit is MINPACK's
 * Levenberg-Marquardt as scipy.optimize.leastsq runs it for the reference
 * (_ROFL_with_jacobi.py:472-486): forward differences, or with grad_mode
 * the reference's own Jacobian (lmder); ftol = xtol = 1.49012e-8, at most
 * 150 evaluations.  Pixels with d_mask[p] == 0 (d_mask may be null) get
 * NaN.  When n_unconverged is non-null the call synchronises and stores
 * the number of pixels that stopped at the evaluation limit (MINPACK's
 * info 5), which the reference passes on silently.
 */
int fpgb_rofl_device(const double *d_data, int64_t n_pix, int64_t n_rot, double tilt_angle,
                     double gain, double dir_offset, int grad_mode,
                     const unsigned char *d_mask, double *d_out, int64_t *n_unconverged,
                     void *stream);

/* Release the library's cached device pool on the current device.  The pool
 * keeps device buffers per (stream, calling host thread) between calls of the
 * host-buffer entry points and of device entry points given no workspace;
 * this frees all of them (after synchronising the device), so it must not
 * run while another thread is inside a call of this library. */
int fpgb_release_pool(void);

/* Release the buffers the calling host thread holds in that pool on the
 * current device (synchronises the device first).  A thread that has made
 * its last call of this library, e.g. a serving worker about to end, frees
 * its share without touching other threads' buffers.  No counterpart in the
 * reference (whose calls allocate and free host memory per call). */
int fpgb_release_thread_pool(void);

#ifdef __cplusplus
}
#endif

#endif /* FASTPLI_GB300_H_ */
