/*
 * TEST INFRASTRUCTURE ONLY.  C-ABI harness around the reference's own,
 * unmodified C++ classes PliGenerator (src/simulation/generator.hpp:16) and
 * PliSimulator (src/simulation/simulator.hpp:14).  Built by oracle/Makefile
 * against the reference sources in place into oracle/_ref/libpliref.so; it is
 * used to pin the C restatement (oracle/pli_oracle.c) and to generate the
 * golden fixtures under tests/golden/.  It replaces the pybind11 modules
 * (src/simulation/bindings/generator_module.cpp:23-140,
 * src/simulation/bindings/simulator_module.cpp:18-157) with plain pointers so
 * no pybind11/Python build is needed.
 */
#include <atomic>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "simulation/fiber_bundle.hpp"
#include "simulation/generator.hpp"
#include "simulation/setup.hpp"
#include "simulation/simulator.hpp"

std::atomic<long> g_oracle_warn_overlap{0};
std::atomic<long> g_oracle_warn_single_point{0};
std::atomic<long> g_oracle_warn_zero_axis{0};
std::atomic<long> g_oracle_warn_not_normalized{0};
std::atomic<long> g_oracle_warn_empty_light{0};
std::atomic<long> g_oracle_warn_other{0};

static std::string g_err;

static void reset_warnings() {
   g_oracle_warn_overlap = 0;
   g_oracle_warn_single_point = 0;
   g_oracle_warn_zero_axis = 0;
   g_oracle_warn_not_normalized = 0;
   g_oracle_warn_empty_light = 0;
   g_oracle_warn_other = 0;
}

static void read_warnings(long *w) {
   if (!w)
      return;
   w[0] = g_oracle_warn_overlap;
   w[1] = g_oracle_warn_single_point;
   w[2] = g_oracle_warn_zero_axis;
   w[3] = g_oracle_warn_not_normalized;
   w[4] = g_oracle_warn_empty_light;
   w[5] = g_oracle_warn_other;
}

extern "C" {

const char *ref_last_error() { return g_err.c_str(); }

/* Number of property rows run_generation returns: 1 + n_bundles * max_layer. */
int ref_generate(const int64_t *dim, const double *origin, double voxel_size,
                 int64_t n_bundles, const int64_t *bundle_fiber_off,
                 const int64_t *fiber_point_off, const double *points,
                 const int64_t *bundle_layer_off, const double *layer_scale,
                 const double *layer_dn, const double *layer_mu,
                 const char *layer_model, int only_label, int n_threads,
                 int32_t *label_out, float *vector_out, double *props_out,
                 int64_t props_cap, int64_t *n_props_out, long *warn_out) {
   try {
      reset_warnings();
      std::vector<fiber::Bundle> bundles;
      for (int64_t b = 0; b < n_bundles; b++) {
         std::vector<std::vector<double>> fibers;
         for (int64_t f = bundle_fiber_off[b]; f < bundle_fiber_off[b + 1];
              f++) {
            const double *p0 = points + 4 * fiber_point_off[f];
            const double *p1 = points + 4 * fiber_point_off[f + 1];
            fibers.emplace_back(p0, p1);
         }
         std::vector<fiber::layer::Property> props;
         for (int64_t l = bundle_layer_off[b]; l < bundle_layer_off[b + 1];
              l++)
            props.emplace_back(layer_scale[l], layer_dn[l], layer_mu[l],
                               layer_model[l]);
         bundles.emplace_back(fibers, props);
      }
      PliGenerator gen;
      gen.set_omp_num_threads(n_threads);
      gen.SetVolume(vm::Vec3<int64_t>(dim[0], dim[1], dim[2]),
                    vm::Vec3<double>(origin[0], origin[1], origin[2]),
                    voxel_size);
      gen.SetFiberBundles(bundles);
      std::vector<int> *label;
      std::vector<float> *vec;
      std::vector<setup::PhyProps> props;
      std::tie(label, vec, props) = gen.RunTissueGeneration(only_label != 0);
      std::memcpy(label_out, label->data(), label->size() * sizeof(int));
      if (!only_label && vector_out)
         std::memcpy(vector_out, vec->data(), vec->size() * sizeof(float));
      *n_props_out = static_cast<int64_t>(props.size());
      for (size_t i = 0; i < props.size() && (int64_t)i < props_cap; i++) {
         props_out[2 * i + 0] = props[i].dn;
         props_out[2 * i + 1] = props[i].mu;
      }
      delete label;
      delete vec;
      read_warnings(warn_out);
      return 0;
   } catch (const std::exception &e) {
      g_err = e.what();
      return -1;
   }
}

int ref_simulate(const int64_t *dim, const int32_t *label, const float *vec,
                 const double *props, int64_t n_props, double step_size,
                 double light_intensity, double voxel_size, double wavelength,
                 double tissue_refrection, int interp, int untilt_sensor_view,
                 int flip_z, const double *rotations, int64_t n_rot,
                 double theta, double phi, int n_threads, double *image_out,
                 long *warn_out) {
   try {
      reset_warnings();
      setup::Setup s;
      s.step_size = step_size;
      s.light_intensity = light_intensity;
      s.voxel_size = voxel_size;
      s.wavelength = wavelength;
      s.tissue_refrection = tissue_refrection;
      s.interpolate = interp == 0   ? setup::InterpMode::nn
                      : interp == 1 ? setup::InterpMode::lerp
                                    : setup::InterpMode::slerp;
      s.untilt_sensor_view = untilt_sensor_view != 0;
      s.flip_z = flip_z != 0;
      s.filter_rotations.assign(rotations, rotations + n_rot);

      const size_t n = static_cast<size_t>(dim[0] * dim[1] * dim[2]);
      object::container::NpArray<int> lab(
          const_cast<int *>(label), n,
          {(size_t)dim[0], (size_t)dim[1], (size_t)dim[2]});
      object::container::NpArray<float> vf(
          const_cast<float *>(vec), 3 * n,
          {(size_t)dim[0], (size_t)dim[1], (size_t)dim[2], 3});
      std::vector<setup::PhyProps> pp;
      for (int64_t i = 0; i < n_props; i++)
         pp.emplace_back(props[2 * i], props[2 * i + 1]);

      PliSimulator sim;
      sim.set_omp_num_threads(n_threads);
      sim.SetSetup(s);
      auto img = sim.RunSimulation(vm::Vec3<int64_t>(dim[0], dim[1], dim[2]),
                                   lab, vf, pp, setup::Tilting(theta, phi));
      std::memcpy(image_out, img.data(), img.size() * sizeof(double));
      read_warnings(warn_out);
      return 0;
   } catch (const std::exception &e) {
      g_err = e.what();
      return -1;
   }
}
}
