/*
 * pli_oracle.c — TEST INFRASTRUCTURE ONLY (the oracle): a double-precision C
 * restatement of the reference's voxelizer and ray march.  See pli_oracle.h
 * for the contract.  Every function cites the reference lines it follows.
 * Compiled with -ffp-contract=off: no product or sum below may be fused.
 */
#define _GNU_SOURCE
#include "pli_oracle.h"

#include <math.h>
#include <stdatomic.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static _Thread_local char g_err[256];
const char *orc_last_error(void) { return g_err; }

static int fail(const char *msg) {
   snprintf(g_err, sizeof g_err, "%s", msg);
   return -1;
}

/* ---------------------------------------------------------------------------
 * small vector helpers with the reference's summation order
 * (std::inner_product starting from T{}: vemath.hpp:342-344, 404-406)
 * ------------------------------------------------------------------------- */
static inline double dot3(const double *a, const double *b) {
   double s = 0.0;
   s = s + a[0] * b[0];
   s = s + a[1] * b[1];
   s = s + a[2] * b[2];
   return s;
}

/* vm::unit: x * (1.0 / sqrt(|x|^2)) when |x|^2 > 0 (vemath.hpp:390-402) */
static inline void unit3(double *u) {
   double n2 = dot3(u, u);
   if (n2 > 0) {
      double inv = 1.0 / sqrt(n2);
      u[0] *= inv;
      u[1] *= inv;
      u[2] *= inv;
   }
}

/* vm::rot_pi_cases::sin / cos: exact values at multiples of pi/2
 * (vemath.hpp:498-520). */
static double pc_sin(double v) {
   v = fmod(v, 2 * M_PI);
   if (v == 0 || v == M_PI || v == -M_PI)
      return 0;
   else if (v == M_PI_2 || v == -(M_PI + M_PI_2))
      return 1;
   else if (v == M_PI + M_PI_2 || v == -M_PI_2)
      return -1;
   return sin(v);
}
static double pc_cos(double v) {
   v = fmod(v, 2 * M_PI);
   if (v == 0)
      return 1;
   else if (v == M_PI_2 || v == M_PI + M_PI_2 || v == -M_PI_2 ||
            v == -(M_PI + M_PI_2))
      return 0;
   else if (v == M_PI || v == -M_PI)
      return -1;
   return cos(v);
}

/* row-major 3x3 helpers (vemath.hpp:346-363, 536-544) */
static void mat3_mul(const double *A, const double *B, double *R) {
   for (int m = 0; m < 3; m++)
      for (int n = 0; n < 3; n++) {
         double s = 0;
         for (int k = 0; k < 3; k++)
            s += A[3 * m + k] * B[3 * k + n];
         R[3 * m + n] = s;
      }
}
static void mat3_vec(const double *A, const double *v, double *r) {
   double t[3];
   for (int i = 0; i < 3; i++) {
      double s = 0.0;
      s = s + v[0] * A[3 * i + 0];
      s = s + v[1] * A[3 * i + 1];
      s = s + v[2] * A[3 * i + 2];
      t[i] = s;
   }
   r[0] = t[0];
   r[1] = t[1];
   r[2] = t[2];
}
static void rot_zyz_pc(double g, double b, double a, double *R) {
   double cg = pc_cos(g), sg = pc_sin(g);
   double cb = pc_cos(b), sb = pc_sin(b);
   double ca = pc_cos(a), sa = pc_sin(a);
   double Zg[9] = {cg, -sg, 0, sg, cg, 0, 0, 0, 1};
   double Yb[9] = {cb, 0, sb, 0, 1, 0, -sb, 0, cb};
   double Za[9] = {ca, -sa, 0, sa, ca, 0, 0, 0, 1};
   double T[9];
   mat3_mul(Yb, Za, T);
   mat3_mul(Zg, T, R);
}

/* ===========================================================================
 * Voxelizer  (generator.cpp:163-383, 475-526; fiber.cpp:83-99,115-150;
 *             fiber_bundle.cpp:19-30,66,76-92,147-154; aabb.hpp:54-137)
 * ========================================================================= */
typedef struct {
   double min[3], max[3];
} box3;

static void box_empty(box3 *b) {
   for (int i = 0; i < 3; i++) {
      b->min[i] = INFINITY;
      b->max[i] = -INFINITY;
   }
}
static void box_pq(box3 *b, const double *p, const double *q) {
   for (int i = 0; i < 3; i++) {
      if (p[i] < q[i]) {
         b->min[i] = p[i];
         b->max[i] = q[i];
      } else {
         b->min[i] = q[i];
         b->max[i] = p[i];
      }
   }
}
static void box_unite(box3 *b, const box3 *a) {
   for (int i = 0; i < 3; i++) {
      if (a->min[i] < b->min[i])
         b->min[i] = a->min[i];
      if (a->max[i] > b->max[i])
         b->max[i] = a->max[i];
   }
}
static int box_overlap(const box3 *a, const box3 *b) {
   for (int i = 0; i < 3; i++)
      if (a->min[i] >= b->max[i] || a->max[i] <= b->min[i])
         return 0;
   return 1;
}

/* Fiber::CalculateVoi (fiber.cpp:83-99) on transformed points. */
static void fiber_box(const double *xyz, const double *r, int64_t n,
                      box3 *out) {
   box_empty(out);
   if (n == 0)
      return;
   const double lo[3] = {xyz[0] - r[0], xyz[1] - r[0], xyz[2] - r[0]};
   const double hi[3] = {xyz[0] + r[0], xyz[1] + r[0], xyz[2] + r[0]};
   box_pq(out, lo, hi);
   for (int64_t s = 0; s + 1 < n; s++) {
      double rm = r[s] < r[s + 1] ? r[s + 1] : r[s]; /* std::max */
      box3 t;
      box_pq(&t, xyz + 3 * s, xyz + 3 * (s + 1));
      for (int i = 0; i < 3; i++) {
         t.min[i] -= rm;
         t.max[i] += rm;
      }
      box_unite(out, &t);
   }
}

typedef struct {
   int n_layers;
   double scale_sq[16];
   double dn[16], mu[16];
   char model[16];
} layer_set;

int orc_generate(const int64_t *dim, const double *origin, double voxel_size,
                 int64_t n_bundles, const int64_t *bundle_fiber_off,
                 const int64_t *fiber_point_off, const double *points,
                 const int64_t *bundle_layer_off, const double *layer_scale,
                 const double *layer_dn, const double *layer_mu,
                 const char *layer_model, int only_label, int n_threads,
                 int32_t *label_out, float *vector_out, double *props_out,
                 int64_t props_cap, int64_t *n_props_out, long *warn_out) {
   /* SetVolume checks (generator.cpp:49-53,115-117) */
   if (dim[0] <= 0 || dim[1] <= 0 || dim[2] <= 0)
      return fail("dim.global[any] <= 0");
   if (voxel_size <= 0)
      return fail("voxel_size <= 0");

   const int64_t X = dim[0], Y = dim[1], Z = dim[2];
   const int64_t nvox = X * Y * Z;
   const int64_t n_fibers = bundle_fiber_off[n_bundles];
   const int64_t n_points = fiber_point_off[n_fibers];

   /* layers per bundle, sorted by scale (fiber_bundle.cpp:19-30,66,83-86) */
   layer_set *ls = calloc((size_t)(n_bundles > 0 ? n_bundles : 1),
                          sizeof(layer_set));
   int max_layer = 0;
   for (int64_t b = 0; b < n_bundles; b++) {
      int64_t l0 = bundle_layer_off[b], l1 = bundle_layer_off[b + 1];
      int n = (int)(l1 - l0);
      if (n > 16) {
         free(ls);
         return fail("more than 16 layers in a bundle");
      }
      int order[16];
      for (int i = 0; i < n; i++)
         order[i] = i;
      for (int i = 1; i < n; i++) { /* stable insertion sort by scale */
         int k = order[i], j = i - 1;
         while (j >= 0 && layer_scale[l0 + k] < layer_scale[l0 + order[j]]) {
            order[j + 1] = order[j];
            j--;
         }
         order[j + 1] = k;
      }
      ls[b].n_layers = n;
      for (int i = 0; i < n; i++) {
         int64_t l = l0 + order[i];
         char m = layer_model[l];
         if (m != 'b' && m != 'p' && m != 'r') {
            free(ls);
            return fail("Orientation must be \"b\", \"p\", or \"r\"");
         }
         ls[b].scale_sq[i] = layer_scale[l] * layer_scale[l];
         ls[b].dn[i] = layer_dn[l];
         ls[b].mu[i] = layer_mu[l];
         ls[b].model[i] = m;
      }
      if (n > max_layer)
         max_layer = n;
   }

   /* translate (only when origin != 0) then resize by 1/voxel_size
    * (generator.cpp:185-197, fiber.cpp:128-150) */
   double *xyz = malloc(sizeof(double) * 3 * (size_t)(n_points ? n_points : 1));
   double *rad = malloc(sizeof(double) * (size_t)(n_points ? n_points : 1));
   const int translate = origin[0] != 0 || origin[1] != 0 || origin[2] != 0;
   const double f = 1.0 / voxel_size;
   for (int64_t i = 0; i < n_points; i++) {
      for (int c = 0; c < 3; c++) {
         double v = points[4 * i + c];
         if (translate)
            v = v + (-origin[c]);
         xyz[3 * i + c] = v * f;
      }
      rad[i] = points[4 * i + 3] * f;
   }

   box3 *fbox = malloc(sizeof(box3) * (size_t)(n_fibers ? n_fibers : 1));
   box3 *bbox = malloc(sizeof(box3) * (size_t)(n_bundles ? n_bundles : 1));
   for (int64_t fi = 0; fi < n_fibers; fi++) {
      int64_t p0 = fiber_point_off[fi], p1 = fiber_point_off[fi + 1];
      fiber_box(xyz + 3 * p0, rad + p0, p1 - p0, &fbox[fi]);
   }
   for (int64_t b = 0; b < n_bundles; b++) { /* fiber_bundle.cpp:147-154 */
      box_empty(&bbox[b]);
      int64_t f0 = bundle_fiber_off[b], f1 = bundle_fiber_off[b + 1];
      if (f1 > f0)
         bbox[b] = fbox[f0];
      for (int64_t fi = f0; fi < f1; fi++)
         box_unite(&bbox[b], &fbox[fi]);
   }

   box3 vol;
   for (int i = 0; i < 3; i++) {
      vol.min[i] = 0.0;
      vol.max[i] = (double)dim[i];
   }

   float *dist = malloc(sizeof(float) * (size_t)nvox);
   for (int64_t i = 0; i < nvox; i++)
      dist[i] = INFINITY;
   memset(label_out, 0, sizeof(int32_t) * (size_t)nvox);
   if (!only_label)
      memset(vector_out, 0, sizeof(float) * 3 * (size_t)nvox);

   atomic_long w_overlap = 0, w_single = 0, w_layer_over = 0;
   atomic_int flag_overlap = 0;

   int nt = n_threads > 0 ? n_threads : 1;
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
   {
#ifdef _OPENMP
      const int tid = omp_get_thread_num();
      const int nth = omp_get_num_threads();
#else
      const int tid = 0, nth = 1;
#endif
      /* every thread walks all segments in order and owns x % nth == tid
       * (generator.cpp:202-232, 314-317) */
      for (int64_t b = 0; b < n_bundles; b++) {
         if (!box_overlap(&vol, &bbox[b]))
            continue;
         const layer_set *L = &ls[b];
         if (L->n_layers == 0)
            continue;
         const double sq_last = L->scale_sq[L->n_layers - 1];
         const float f_ly_squ = (float)sq_last;
         for (int64_t fi = bundle_fiber_off[b]; fi < bundle_fiber_off[b + 1];
              fi++) {
            int64_t p0 = fiber_point_off[fi], p1 = fiber_point_off[fi + 1];
            if (p1 - p0 <= 1) {
               if (tid == 0)
                  w_single++;
               continue;
            }
            if (!box_overlap(&vol, &fbox[fi]))
               continue;
            for (int64_t s = p0; s + 1 < p1; s++) {
               const double *P = xyz + 3 * s, *Q = xyz + 3 * (s + 1);
               const double r0 = rad[s], r1 = rad[s + 1];
               /* FillVoxelsAroundFiberSegment (generator.cpp:293-305) */
               const double rmax = (r0 < r1 ? r1 : r0) * sqrt(sq_last);
               box3 sb;
               box_pq(&sb, P, Q);
               int64_t lo[3], hi[3];
               for (int i = 0; i < 3; i++) {
                  sb.min[i] -= rmax;
                  sb.max[i] += rmax;
                  if (vol.min[i] > sb.min[i])
                     sb.min[i] = vol.min[i];
                  if (vol.max[i] < sb.max[i])
                     sb.max[i] = vol.max[i];
                  lo[i] = (int64_t)sb.min[i];
                  hi[i] = (int64_t)(sb.max[i] + 0.5);
               }
               double v[3] = {Q[0] - P[0], Q[1] - P[1], Q[2] - P[2]};
               const double c2 = dot3(v, v);
               for (int64_t x = lo[0]; x < hi[0]; x++) {
                  if (x % nth != tid)
                     continue;
                  for (int64_t y = lo[1]; y < hi[1]; y++)
                     for (int64_t z = lo[2]; z < hi[2]; z++) {
                        const double pt[3] = {x + 0.5, y + 0.5, z + 0.5};
                        /* closest point on the segment (generator.cpp:475-494) */
                        double w[3] = {pt[0] - P[0], pt[1] - P[1], pt[2] - P[2]};
                        double c1 = dot3(w, v);
                        double cl[3], t;
                        if (c1 < 0) {
                           cl[0] = P[0]; cl[1] = P[1]; cl[2] = P[2];
                           t = 0;
                        } else if (c2 <= c1) {
                           cl[0] = Q[0]; cl[1] = Q[1]; cl[2] = Q[2];
                           t = 1;
                        } else {
                           double bq = c1 / c2;
                           cl[0] = P[0] + v[0] * bq;
                           cl[1] = P[1] + v[1] * bq;
                           cl[2] = P[2] + v[2] * bq;
                           t = bq;
                        }
                        double d[3] = {cl[0] - pt[0], cl[1] - pt[1],
                                       cl[2] - pt[2]};
                        const float dist_squ = (float)dot3(d, d);
                        /* Fiber::CalcRadius (fiber.cpp:115-120) */
                        const double rr = r0 * (1 - t) + r1 * t;
                        const float r_sqr = (float)(rr * rr);
                        if (dist_squ > f_ly_squ * r_sqr)
                           continue;
                        const int64_t ind = x * Y * Z + y * Z + z;
                        if (dist[ind] >= dist_squ) {
                           /* std::lower_bound over scale^2 (generator.cpp:345-349) */
                           const double qv = (double)(dist_squ / r_sqr);
                           int ly = 0;
                           while (ly < L->n_layers && L->scale_sq[ly] < qv)
                              ly++;
                           const int new_label =
                               ly + 1 + (int)b * max_layer;
                           if (!atomic_load(&flag_overlap) &&
                               label_out[ind] != 0 &&
                               abs(label_out[ind] - new_label) >= max_layer) {
                              if (!atomic_exchange(&flag_overlap, 1))
                                 w_overlap++;
                           }
                           dist[ind] = dist_squ;
                           label_out[ind] = new_label;
                           if (!only_label) {
                              double nv[3] = {0, 0, 0};
                              char m = 'b';
                              if (ly < L->n_layers)
                                 m = L->model[ly];
                              else
                                 w_layer_over++;
                              if (m == 'r') {
                                 nv[0] = pt[0] - cl[0];
                                 nv[1] = pt[1] - cl[1];
                                 nv[2] = pt[2] - cl[2];
                                 unit3(nv);
                              } else if (m == 'p') {
                                 nv[0] = v[0]; nv[1] = v[1]; nv[2] = v[2];
                                 unit3(nv);
                              }
                              vector_out[3 * ind + 0] = (float)nv[0];
                              vector_out[3 * ind + 1] = (float)nv[1];
                              vector_out[3 * ind + 2] = (float)nv[2];
                           }
                        }
                     }
               }
            }
         }
      }
   }

   /* GetPropertyList (generator.cpp:496-526) */
   int64_t n_props = n_bundles * max_layer + 1;
   *n_props_out = n_props;
   for (int64_t i = 0; i < n_props && i < props_cap; i++) {
      props_out[2 * i] = 0;
      props_out[2 * i + 1] = 0;
   }
   for (int64_t b = 0; b < n_bundles; b++)
      for (int l = 0; l < ls[b].n_layers; l++) {
         int64_t id = 1 + l + b * max_layer;
         if (id >= props_cap)
            continue;
         props_out[2 * id + 1] = ls[b].mu[l];
         props_out[2 * id] = ls[b].model[l] == 'b' ? 0 : ls[b].dn[l];
      }

   if (warn_out) {
      warn_out[0] = w_overlap;
      warn_out[1] = w_single;
      warn_out[2] = 0;
      warn_out[3] = 0;
      warn_out[4] = 0;
      warn_out[5] = w_layer_over;
   }
   free(dist);
   free(fbox);
   free(bbox);
   free(xyz);
   free(rad);
   free(ls);
   return 0;
}

/* ===========================================================================
 * Ray march  (simulator.cpp:131-411, 417-579, 585-773)
 * ========================================================================= */
typedef struct {
   int64_t X, Y, Z;
   const int32_t *label;
   const float *vec;
   int flip_z;
} field;

static inline int64_t llfloor(double v) { return (int64_t)floor(v); }
static inline int64_t llceil(double v) { return (int64_t)ceil(v); }

/* GetLabel (simulator.cpp:425-443) */
static inline int get_label(const field *F, int64_t x, int64_t y, int64_t z) {
   if (F->flip_z)
      z = F->Z - 1 - z;
   if (x < 0 || x >= F->X || y < 0 || y >= F->Y || z < 0 || z >= F->Z)
      return 0;
   return F->label[x * F->Y * F->Z + y * F->Z + z];
}
/* GetVec (simulator.cpp:557-579) */
static inline void get_vec(const field *F, int64_t x, int64_t y, int64_t z,
                           double *o) {
   if (F->flip_z)
      z = F->Z - 1 - z;
   const float *p = F->vec + 3 * (x * F->Y * F->Z + y * F->Z + z);
   o[0] = p[0];
   o[1] = p[1];
   o[2] = p[2];
}
static inline int is_zero(const double *v) {
   return v[0] == 0 && v[1] == 0 && v[2] == 0;
}
/* LinearOrientationInterpolation + VectorOrientationAddition
 * (simulator.cpp:449-471) */
static void lerp_or(const double *v, const double *u, double t, double *o) {
   if (is_zero(v)) {
      o[0] = u[0]; o[1] = u[1]; o[2] = u[2];
      return;
   }
   if (is_zero(u)) {
      o[0] = v[0]; o[1] = v[1]; o[2] = v[2];
      return;
   }
   double a[3] = {v[0] * (1 - t), v[1] * (1 - t), v[2] * (1 - t)};
   double b[3] = {u[0] * t, u[1] * t, u[2] * t};
   if (dot3(a, b) >= 0) {
      o[0] = a[0] + b[0]; o[1] = a[1] + b[1]; o[2] = a[2] + b[2];
   } else {
      o[0] = a[0] - b[0]; o[1] = a[1] - b[1]; o[2] = a[2] - b[2];
   }
}
/* SphericalInterpolation (simulator.cpp:473-494) */
static void slerp_or(const double *v, const double *u_in, double t,
                     double *o) {
   if (is_zero(v)) {
      o[0] = u_in[0]; o[1] = u_in[1]; o[2] = u_in[2];
      return;
   }
   if (is_zero(u_in)) {
      o[0] = v[0]; o[1] = v[1]; o[2] = v[2];
      return;
   }
   double u[3] = {u_in[0], u_in[1], u_in[2]};
   if (dot3(v, u) < 0) {
      u[0] = -u[0]; u[1] = -u[1]; u[2] = -u[2];
   }
   double d[3] = {v[0] - u[0], v[1] - u[1], v[2] - u[2]};
   if (dot3(d, d) < 1e-12) {
      o[0] = v[0]; o[1] = v[1]; o[2] = v[2];
      return;
   }
   const double th = acos(dot3(v, u) / (sqrt(dot3(v, v)) * sqrt(dot3(u, u))));
   const double s = sin(th), sa = sin((1 - t) * th), sb = sin(t * th);
   for (int i = 0; i < 3; i++)
      o[i] = v[i] * sa / s + u[i] * sb / s;
}

/* GetVec with interpolation (simulator.cpp:496-555) */
static void get_vec_interp(const field *F, double x, double y, double z,
                           int mode, double *o) {
   if (mode == 0) {
      get_vec(F, llfloor(x), llfloor(y), llfloor(z), o);
      return;
   }
   const int label = get_label(F, llfloor(x), llfloor(y), llfloor(z));
   if (label == 0) {
      o[0] = o[1] = o[2] = 0;
      return;
   }
#define CLAMP(v, hi) ((v) < 0 ? 0 : ((v) > (hi) ? (hi) : (v)))
   const int64_t x0 = CLAMP(llfloor(x - 0.5), F->X - 1);
   const int64_t y0 = CLAMP(llfloor(y - 0.5), F->Y - 1);
   const int64_t z0 = CLAMP(llfloor(z - 0.5), F->Z - 1);
   const int64_t x1 = CLAMP(llceil(x - 0.5), F->X - 1);
   const int64_t y1 = CLAMP(llceil(y - 0.5), F->Y - 1);
   const int64_t z1 = CLAMP(llceil(z - 0.5), F->Z - 1);
#undef CLAMP
   if (x0 == x1 && y0 == y1 && z0 == z1) {
      get_vec(F, x0, y0, z0, o);
      return;
   }
   double xd = (x - (double)x0 - 0.5) / (double)(x1 - x0);
   double yd = (y - (double)y0 - 0.5) / (double)(y1 - y0);
   double zd = (z - (double)z0 - 0.5) / (double)(z1 - z0);
   if (x0 == x1)
      xd = 0;
   if (y0 == y1)
      yd = 0;
   if (z0 == z1)
      zd = 0;
   double c[8][3];
   const int64_t xs[2] = {x0, x1}, ys[2] = {y0, y1}, zs[2] = {z0, z1};
   /* index bits: (x, y, z) -> c[x + 2y + 4z] */
   for (int k = 0; k < 8; k++) {
      int64_t xi = xs[k & 1], yi = ys[(k >> 1) & 1], zi = zs[(k >> 2) & 1];
      get_vec(F, xi, yi, zi, c[k]);
      double m = get_label(F, xi, yi, zi) == label;
      c[k][0] *= m;
      c[k][1] *= m;
      c[k][2] *= m;
   }
   void (*ip)(const double *, const double *, double, double *) =
       mode == 2 ? slerp_or : lerp_or;
   double c00[3], c01[3], c10[3], c11[3], c0[3], c1[3];
   ip(c[0], c[1], xd, c00); /* c000, c100 */
   ip(c[4], c[5], xd, c01); /* c001, c101 */
   ip(c[2], c[3], xd, c10); /* c010, c110 */
   ip(c[6], c[7], xd, c11); /* c011, c111 */
   ip(c00, c10, yd, c0);
   ip(c01, c11, yd, c1);
   ip(c0, c1, zd, o);
}

int orc_simulate(const int64_t *dim, const int32_t *label, const float *vec,
                 const double *props, int64_t n_props, double step_size,
                 double light_intensity, double voxel_size, double wavelength,
                 double tissue_refrection, int interp, int untilt_sensor_view,
                 int flip_z, const double *rotations, int64_t n_rot,
                 double theta, double phi, int n_threads, double *image_out,
                 long *warn_out) {
   /* Setup::Check (setup.hpp:48-71) */
   if (step_size <= 0)
      return fail("step_size <= 0");
   if (light_intensity < 0)
      return fail("light intensity < 0");
   if (voxel_size <= 0)
      return fail("voxel_size <= 0");
   if (wavelength <= 0)
      return fail("wavelength <= 0");
   if (tissue_refrection < 1)
      return fail("tissue_refrection < 1");
   if (n_rot <= 0)
      return fail("filter_rotations is empty: []");
   if (interp < 0 || interp > 2)
      return fail("Only NN, Lerp or Slerp are supported");
   const int64_t X = dim[0], Y = dim[1], Z = dim[2];
   if (X <= 0 || Y <= 0 || Z <= 0)
      return fail("global_dim[any] <= 0");
   /* CheckInput (simulator.cpp:139-175) */
   const int64_t nvox = X * Y * Z;
   int lmin = 0x7fffffff, lmax = -0x7fffffff - 1;
   for (int64_t i = 0; i < nvox; i++) {
      if (label[i] < lmin)
         lmin = label[i];
      if (label[i] > lmax)
         lmax = label[i];
   }
   if (lmin < 0 || lmax < 0)
      return fail("label < 0 detected");
   if ((int64_t)lmax >= n_props)
      return fail("label exceed properties.size()");
   if (props[0] != 0)
      return fail("background birefringence has to be 0");
   for (int64_t i = 0; i < n_props; i++)
      if (props[2 * i + 1] < 0)
         return fail("mu < 0");

   const double lambda = wavelength * 1e-9;
   const double thickness = voxel_size * 1e-6 * step_size;

   /* initial Stokes vector PolX(1) then lambda/4 retarder
    * (simulator.cpp:28-56, 203-214): (I/2, 0, 0, -I/2) */
   double s_init[4];
   {
      const double Px[16] = {0.5, 0.5, 0, 0, 0.5, 0.5, 0, 0,
                             0, 0, 0, 0, 0, 0, 0, 0};
      const double cb = pc_cos(M_PI_2), sb = pc_sin(M_PI_2);
      const double cr = pc_cos(-M_PI_2), sr = pc_sin(-M_PI_2);
      const double Mr[16] = {1, 0, 0, 0,
                             0, pow(cb, 2) + cr * pow(sb, 2),
                             (1 - cr) * sb * cb, -sr * sb,
                             0, (1 - cr) * sb * cb,
                             pow(sb, 2) + cr * pow(cb, 2), sr * cb,
                             0, sr * sb, -sr * cb, cr};
      double s0[4] = {light_intensity, 0, 0, 0}, s1[4];
      for (int i = 0; i < 4; i++) {
         double a = 0;
         for (int k = 0; k < 4; k++)
            a = a + s0[k] * Px[4 * i + k];
         s1[i] = a;
      }
      for (int i = 0; i < 4; i++) {
         double a = 0;
         for (int k = 0; k < 4; k++)
            a = a + s1[k] * Mr[4 * i + k];
         s_init[i] = a;
      }
   }

   double rot[9];
   rot_zyz_pc(phi, theta, -phi, rot);
   const double dir[3] = {pc_cos(phi) * pc_sin(theta),
                          pc_sin(phi) * pc_sin(theta), pc_cos(theta)};
   const double step[3] = {dir[0] * step_size, dir[1] * step_size,
                           dir[2] * step_size};
   const double shift[3] = {dir[0] / cos(theta) * (double)Z,
                            dir[1] / cos(theta) * (double)Z,
                            dir[2] / cos(theta) * (double)Z};

   /* tilted-view geometry (simulator.cpp:614-719) */
   double rt[9], rti[9], pc[3], pt[3], p1[3], p2[3], A = 0, B = 0, C = 0,
                                                      Dd = 0;
   if (!untilt_sensor_view) {
      const double ang = asin(sin(-theta) * tissue_refrection);
      rot_zyz_pc(phi, ang, -phi, rt);
      rot_zyz_pc(phi, -ang, -phi, rti);
      pc[0] = (double)X * 0.5;
      pc[1] = (double)Y * 0.5;
      pc[2] = (double)Z * 0.5;
      double t0[3] = {-pc[0], -pc[1], pc[2]};
      double e1[3] = {1, 0, 0}, e2[3] = {0, 1, 0};
      mat3_vec(rt, t0, pt);
      mat3_vec(rt, e1, p1);
      mat3_vec(rt, e2, p2);
      A = p1[0];
      B = p2[0];
      C = p1[1];
      Dd = p2[1];
   }

   field F = {X, Y, Z, label, vec, flip_z};
   const int64_t n_rays = X * Y;
   atomic_long w_zero = 0, w_norm = 0;
   const int nt = n_threads > 0 ? n_threads : 1;
   double *sv = NULL;
   (void)sv;

#ifdef _OPENMP
#pragma omp parallel for schedule(guided) num_threads(nt)
#endif
   for (int64_t ray = 0; ray < n_rays; ray++) {
      const int64_t cx = ray / Y, cy = ray % Y;
      double pos[3];
      if (untilt_sensor_view) { /* simulator.cpp:721-773 */
         pos[0] = (cx + 0.5) - 0.5 * shift[0];
         pos[1] = (cy + 0.5) - 0.5 * shift[1];
         pos[2] = 0.0;
      } else {
         const double e = cx + 0.5 - pc[0] - pt[0];
         const double f = cy + 0.5 - pc[1] - pt[1];
         const double D = A * Dd - C * B;
         const double Ds = e * Dd - f * B;
         const double Dt = A * f - C * e;
         const double s = Ds / D, t = Dt / D;
         double pp[3], rel[3], ts[3];
         for (int i = 0; i < 3; i++)
            pp[i] = pc[i] + pt[i] + p1[i] * s + p2[i] * t;
         for (int i = 0; i < 3; i++)
            rel[i] = pp[i] - pc[i];
         mat3_vec(rti, rel, ts);
         for (int i = 0; i < 3; i++)
            ts[i] = ts[i] + pc[i];
         pos[0] = ts[0] - shift[0];
         pos[1] = ts[1] - shift[1];
         pos[2] = 0.0;
      }
      for (int i = 0; i < 3; i++) /* simulator.cpp:230-231 */
         pos[i] = pos[i] + step[i] * 0.5;

      double S[64][4];
      double (*s_vec)[4] = S;
      double *heap = NULL;
      if (n_rot > 64) {
         heap = malloc(sizeof(double) * 4 * (size_t)n_rot);
         s_vec = (double(*)[4])heap;
      }
      for (int64_t r = 0; r < n_rot; r++)
         for (int k = 0; k < 4; k++)
            s_vec[r][k] = s_init[k];

      for (; llfloor(pos[2]) >= 0 && llfloor(pos[2]) < Z;
           pos[0] = pos[0] + step[0], pos[1] = pos[1] + step[1],
           pos[2] = pos[2] + step[2]) {
         const int lab =
             get_label(&F, llfloor(pos[0]), llfloor(pos[1]), llfloor(pos[2]));
         const double dn = props[2 * lab];
         const double mu = props[2 * lab + 1] * 1e3;
         const double att = exp(-mu * thickness);
         if (dn == 0 || lab == 0) {
            if (mu == 0)
               continue;
            for (int64_t r = 0; r < n_rot; r++)
               for (int k = 0; k < 4; k++)
                  s_vec[r][k] *= att;
            continue;
         }
         double v[3];
         get_vec_interp(&F, pos[0], pos[1], pos[2], interp, v);
         if (is_zero(v)) {
            w_zero++;
            continue;
         }
         if (dot3(v, v) - 1 > 1e-5)
            w_norm++;
         const double d_rel = dn * 4.0 * thickness / lambda * sqrt(dot3(v, v));
         if (theta != 0)
            mat3_vec(rot, v, v);
         const double alpha = asin(v[2] / sqrt(dot3(v, v)));
         const double ret = M_PI_2 * d_rel * pow(cos(alpha), 2.0);
         const double sin_r = sin(ret), cos_r = cos(ret);
         const double phii = atan2(v[1], v[0]);
         for (int64_t r = 0; r < n_rot; r++) {
            const double beta = 2 * (rotations[r] - phii);
            const double sin_b = sin(-beta), cos_b = cos(-beta);
            double *s = s_vec[r];
            const double a1 = s[1] * cos_b - s[2] * sin_b;
            const double c1 = s[1] * sin_b + s[2] * cos_b;
            const double b1 = c1 * cos_r + s[3] * sin_r;
            const double n1 = a1 * cos_b + b1 * sin_b;
            const double n2 = -a1 * sin_b + b1 * cos_b;
            const double n3 = -c1 * sin_r + s[3] * cos_r;
            s[1] = n1;
            s[2] = n2;
            s[3] = n3;
            for (int k = 0; k < 4; k++)
               s[k] *= att;
         }
      }
      /* analyser PolY(1): s0*0.5 + s1*(-0.5) (simulator.cpp:346-362) */
      for (int64_t r = 0; r < n_rot; r++) {
         double a = 0;
         a = a + s_vec[r][0] * 0.5;
         a = a + s_vec[r][1] * -0.5;
         a = a + s_vec[r][2] * 0.0;
         a = a + s_vec[r][3] * 0.0;
         image_out[(cx * Y + cy) * n_rot + r] = a;
      }
      free(heap);
   }

   if (warn_out) {
      warn_out[0] = 0;
      warn_out[1] = 0;
      warn_out[2] = w_zero;
      warn_out[3] = w_norm;
      warn_out[4] = 0;
      warn_out[5] = 0;
   }
   return 0;
}
