/*
 * pli_oracle — TEST INFRASTRUCTURE, not the product.
 *
 * A plain-C, double-precision restatement of fastpli's simulation forward
 * model: the PliGenerator voxelizer (src/simulation/generator.cpp:163-383,
 * 475-526) and the PliSimulator ray march (src/simulation/simulator.cpp:
 * 28-56, 131-411, 417-579, 585-773), with the arithmetic order of the
 * reference kept operation for operation so that labels and vectors come out
 * bit-identical and images agree to rounding.  Only tests/, the smoke check
 * and bench.py's CPU-baseline leg call it, always as the checker.
 *
 * Parity of this restatement is pinned against the reference's own C++
 * (built by `make -C oracle ref` into oracle/_ref) and against the golden
 * fixtures under tests/golden/ that the reference produced.
 *
 * Warning counters (long[6]) follow the reference's PyErr_WarnEx sites:
 *   [0] "objects overlap"                 generator.cpp:357
 *   [1] "fiber object with only single point"  generator.cpp:215
 *   [2] "optical_axis is 0 for tissue > 0"     simulator.cpp:294
 *   [3] "optical_axis not normalized"          simulator.cpp:300
 *   [4] "light_positions is empty"             simulator.cpp:715,769
 *   [5] voxels whose layer quotient exceeds the outermost layer (the
 *       reference reads past its layer table there, generator.cpp:345-366;
 *       this restatement writes a zero vector and counts them)
 */
#ifndef ORACLE_PLI_ORACLE_H_
#define ORACLE_PLI_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Returns 0 on success, -1 on an argument error (message in
 * orc_last_error()).  Fibers: points[n_points][4] = (x, y, z, r) in µm,
 * fiber f of the flat list owns points [fiber_point_off[f],
 * fiber_point_off[f+1]); bundle b owns fibers [bundle_fiber_off[b],
 * bundle_fiber_off[b+1]) and layers [bundle_layer_off[b],
 * bundle_layer_off[b+1]) given as (scale, dn, mu, model char 'b'|'p'|'r').
 * Outputs: label[X*Y*Z] int32, vector[X*Y*Z*3] float (skipped when
 * only_label), props[(1 + n_bundles*max_layer) * 2] as (dn, mu) rows. */
int orc_generate(const int64_t *dim, const double *origin, double voxel_size,
                 int64_t n_bundles, const int64_t *bundle_fiber_off,
                 const int64_t *fiber_point_off, const double *points,
                 const int64_t *bundle_layer_off, const double *layer_scale,
                 const double *layer_dn, const double *layer_mu,
                 const char *layer_model, int only_label, int n_threads,
                 int32_t *label_out, float *vector_out, double *props_out,
                 int64_t props_cap, int64_t *n_props_out, long *warn_out);

/* interp: 0 = NN, 1 = Lerp, 2 = Slerp.  image_out[X*Y*n_rot] float64. */
int orc_simulate(const int64_t *dim, const int32_t *label, const float *vec,
                 const double *props, int64_t n_props, double step_size,
                 double light_intensity, double voxel_size, double wavelength,
                 double tissue_refrection, int interp, int untilt_sensor_view,
                 int flip_z, const double *rotations, int64_t n_rot,
                 double theta, double phi, int n_threads, double *image_out,
                 long *warn_out);

const char *orc_last_error(void);

#ifdef __cplusplus
}
#endif

#endif
