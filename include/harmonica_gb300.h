/*
 * harmonica_gb300 — C ABI of the GB300 (sm_103a) prism gravity forward model.
 *
 * Every entry point takes plain pointers and sizes; no C++ or torch types
 * cross this boundary and no exception escapes it.  Unless stated otherwise,
 * array arguments are DEVICE pointers owned by the caller, the work is queued
 * asynchronously on `stream` (a cudaStream_t, NULL = legacy default stream),
 * and the return value is HG_OK or a negative HG_ERR_* code whose message is
 * available from hg_last_error() on the calling thread.
 *
 * Field codes and bit masks (harmonica FIELDS, src/harmonica/_forward/prisms/gravity.py:37-48):
 *   0 potential  (J/kg)     bit 1<<0
 *   1 g_e        (mGal)     bit 1<<1
 *   2 g_n        (mGal)     bit 1<<2
 *   3 g_z        (mGal, downward)   bit 1<<3
 *   4 g_ee       (Eotvos)   bit 1<<4
 *   5 g_nn       (Eotvos)   bit 1<<5
 *   6 g_zz       (Eotvos)   bit 1<<6
 *   7 g_en       (Eotvos)   bit 1<<7
 *   8 g_ez       (Eotvos, easting-downward)   bit 1<<8
 *   9 g_nz       (Eotvos, northing-downward)  bit 1<<9
 * Outputs carry harmonica's units and signs (gravity.py:227-236).  With more
 * than one bit set, `out` holds one row of n_obs values per requested field,
 * in increasing field-code order.
 */
#ifndef HARMONICA_GB300_H
#define HARMONICA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HG_OK 0
#define HG_ERR_INVALID (-1)
#define HG_ERR_CUDA (-2)

#define HG_FIELD_MASK_ALL 0x3FFu

/* Library version (major*10000 + minor*100 + patch). */
int hg_version(void);

/* Message of the last failed call on this thread ("" if none). */
const char *hg_last_error(void);

/*
 * Pack an (n_prisms, 6) row-major array [w, e, s, n, b, t] and a density
 * vector into the structure-of-arrays layout the forward kernels read:
 * 7 rows (w, e, s, n, b, t, rho) of `prism_stride` doubles each.
 * Replaces the host-side reshaping of harmonica's prism_gravity
 * (np.atleast_2d / ravel, gravity.py:200-205).
 */
int hg_pack_prisms(const double *prisms_aos, const double *density, int64_t n_prisms,
                   double *prisms_soa, int64_t prism_stride, void *stream);

/*
 * Top and bottom of a layer of prisms from its surface and reference
 * (replaces the host update in DatasetAccessorPrismLayer.update_top_bottom,
 * src/harmonica/_forward/prisms/layer.py:264-312): element-wise, top = the
 * reference where the surface is below it, else the surface; bottom the
 * other one.  reference: n doubles (device), or NULL to use reference_value
 * everywhere.  All arrays in device memory; asynchronous on `stream`.
 */
int hg_layer_top_bottom(const double *surface, const double *reference, double reference_value,
                        int64_t n, double *top, double *bottom, void *stream);

/*
 * Bytes of device workspace hg_prism_forward needs for this problem
 * (0 when the launch writes `out` directly).
 */
int hg_prism_forward_workspace(int64_t n_obs, int64_t n_prisms, uint32_t field_mask,
                               size_t *bytes);

/*
 * All-pairs prism gravity: out[f][i] = sum over prisms j of the field f of
 * prism j at observation point i.  Replaces harmonica's hot loop
 * jit_prism_gravity (src/harmonica/_forward/prisms/gravity.py:489-545) with
 * the null-prism discard of _discard_null_prisms (gravity.py:452-486) fused
 * (prisms with w == e, s == n, b == t or rho == 0 contribute nothing) and the
 * singular-point scan of _check_singular_points (gravity.py:239-449) fused:
 * if `singular_flag` is not NULL, *singular_flag is OR-ed with 1 when any
 * observation point lies on a singular edge or vertex of any prism (null
 * prisms included) for a requested tensor field; the caller zeroes it first.
 * Tensor values at singular points are NaN, as in the reference.
 *   obs_e/n/u    : n_obs doubles each
 *   prisms_soa   : 7 rows of prism_stride doubles (see hg_pack_prisms)
 *   out          : popcount(field_mask) rows of n_obs doubles
 *   workspace    : hg_prism_forward_workspace() bytes, or NULL to let the
 *                  library allocate it on `stream` (cudaMallocAsync).
 */
int hg_prism_forward(const double *obs_e, const double *obs_n, const double *obs_u, int64_t n_obs,
                     const double *prisms_soa, int64_t prism_stride, int64_t n_prisms,
                     uint32_t field_mask, double *out, int32_t *singular_flag, void *workspace,
                     size_t workspace_bytes, void *stream);

/*
 * hg_prism_forward for callers that cannot allocate device memory (no
 * counterpart in the reference: harmonica never touches device memory).
 * Frameworks that own the device pool, latency-critical loops that must not
 * allocate mid-step, and plugins with a fixed GPU memory budget can neither
 * pass hg_prism_forward a workspace nor let it allocate one.  This entry point
 * computes exactly what hg_prism_forward computes (same arguments minus the
 * workspace) and calls no cudaMalloc/cudaFree: its scratch for partial sums
 * is a fixed 8 MiB array in the library's device image, held by every GPU
 * that loads the library until the process exits.
 *   - When the usual split of the prisms into chunks would need more than
 *     8 MiB of partial sums (n_chunks x fields x n_obs doubles), the prisms
 *     are split into fewer, longer chunks, down to a single chunk, which
 *     needs no scratch: no problem is rejected for its size.  Results then
 *     differ from hg_prism_forward's only by the order in which the chunk
 *     sums are added; many fields at once over tens of thousands of points
 *     run with less parallelism.
 *   - The first call on each device looks up the array's device address
 *     (cudaGetSymbolAddress) with that device current and keeps it for the
 *     life of the process; make that first call before any stream capture,
 *     and do not reset the device (cudaDeviceReset) while using this entry.
 *   - All calls on a device share the one array and it keeps the last call's
 *     contents (nothing in it needs to start at zero).  Calls that overlap on
 *     the GPU (e.g. on two streams at once) race on it: serialise them.
 */
int hg_prism_forward_noalloc(const double *obs_e, const double *obs_n, const double *obs_u,
                             int64_t n_obs, const double *prisms_soa, int64_t prism_stride,
                             int64_t n_prisms, uint32_t field_mask, double *out,
                             int32_t *singular_flag, void *stream);

/* Bytes of device workspace hg_layer_forward needs for this problem. */
int hg_layer_forward_workspace(int64_t n_obs, int64_t n_east, int64_t n_north,
                               uint32_t field_mask, size_t *bytes);

/*
 * Prism-layer forward.  Replaces the loop of _forward_gravity_prism_layer
 * (src/harmonica/_forward/prisms/layer.py:522-633) behind
 * DatasetAccessorPrismLayer.gravity (layer.py:314-433): prism boundaries are
 * generated from the regular grid of centres +- half the spacing, and prisms
 * with zero or NaN density, thickness below `thickness_threshold`, or NaN top
 * or bottom are skipped (layer.py:596-607).
 *   centre_e     : n_east easting centres (regular, n_east >= 2)
 *   centre_n     : n_north northing centres (regular, n_north >= 2)
 *   bottom, top, density : (n_north, n_east) row-major
 */
int hg_layer_forward(const double *obs_e, const double *obs_n, const double *obs_u, int64_t n_obs,
                     const double *centre_e, int64_t n_east, const double *centre_n,
                     int64_t n_north, const double *bottom, const double *top,
                     const double *density, double thickness_threshold, uint32_t field_mask,
                     double *out, void *workspace, size_t workspace_bytes, void *stream);

/*
 * ---------------------------------------------------------------------------
 * Batched forward: many independent problems (each its own points, prisms
 * and ONE field) in one persistent launch per field present.  Replaces a
 * Python loop of harmonica prism_gravity calls (gravity.py:51-236), one per
 * problem, with launches whose work items (problem, 128-point tile, prism
 * chunk) are pulled from a device queue by a persistent grid running that
 * field's specialised kernel; each point's chunks are added in fixed order,
 * so every result is bitwise the same alone and in any batch.
 */
typedef struct hg_problem {
  const double *obs_e;       /* n_obs (device) */
  const double *obs_n;
  const double *obs_u;
  int64_t n_obs;
  const double *prisms_soa;  /* 7 rows of prism_stride (hg_pack_prisms layout) */
  int64_t prism_stride;
  int64_t n_prisms;
  int32_t field;             /* field code 0..9 */
  int32_t check_singular;    /* 1: OR 1 into *singular_flag on a singular point */
  double *out;               /* n_obs (device), harmonica units */
  int32_t *singular_flag;    /* device int32 or NULL */
} hg_problem;

typedef struct hg_batch hg_batch; /* opaque plan */

/*
 * Build the work list of a batch (host work + two small device copies; the
 * plan keeps device pointers of the problems, which must stay valid until
 * hg_batch_destroy).  chunk_prisms <= 0 and n_ctas <= 0 choose automatically
 * (about 16 work items per CTA; per field, one full wave of that field's
 * kernel).  A given n_ctas applies to every field's launch; every field runs
 * 128 points per CTA.
 */
int hg_batch_create(const hg_problem *problems, int64_t n_problems, int64_t chunk_prisms,
                    int32_t n_ctas, hg_batch **batch);

/*
 * Shape of the work of one field in a batch (chosen per field by the
 * autotuner of harmonica_gb300.batch):
 *   chunk_prisms   : prisms per work item, rounded up to whole prism tiles
 *                    (0: about 16 work items per CTA of the field's launch)
 *   points_per_cta : observation points per CTA and per work item, which is
 *                    also the prisms staged per shared-memory tile: 64 or 128
 *                    (0: 128)
 *   n_ctas         : CTAs of the field's persistent launch (0: one full wave)
 */
typedef struct hg_batch_shape {
  int64_t chunk_prisms;
  int32_t points_per_cta;
  int32_t n_ctas;
} hg_batch_shape;

/*
 * hg_batch_create with one shape per field code (shapes[0..9]); a problem's
 * result is bitwise the same alone and in any batch built with the same
 * shape for its field.
 */
int hg_batch_create_shaped(const hg_problem *problems, int64_t n_problems,
                           const hg_batch_shape *shapes, hg_batch **batch);

/* Bytes of device workspace hg_batch_run needs. */
int hg_batch_workspace(const hg_batch *batch, size_t *bytes);

/* Work items, persistent CTAs (of the g_z launch, or the given count) and prism-point pairs. */
int hg_batch_info(const hg_batch *batch, int64_t *n_items, int64_t *n_ctas, double *pairs);

/*
 * Run the batch on `stream`: one memset, one launch per field present (two
 * for the potential, its edge-log and face terms, with a counter reset
 * between them) and one reduction launch, no allocation and no host
 * synchronisation
 * (capturable in a CUDA graph; replays recompute from the current contents
 * of the problems' input buffers).
 */
int hg_batch_run(const hg_batch *batch, void *workspace, size_t workspace_bytes, void *stream);

/* Free a plan (device work list included). */
int hg_batch_destroy(hg_batch *batch);

/*
 * ---------------------------------------------------------------------------
 * Rounds for continuous batching (a serving loop admits requests while
 * earlier ones are on the GPU and launches a round of work items from many
 * requests at a time).  The caller keeps, in device memory, a table of
 * hg_problem_plan entries and, per round, a list of hg_work_item; every
 * item (problem, 128-point tile, prism chunk) writes its partial sums to
 * problem.partials[chunk * n_obs + point].  hg_round_reduce then adds the
 * chunks of finished problems in fixed order into problem.out, so a result
 * does not depend on which rounds or neighbours its items ran with.
 */
typedef struct hg_problem_plan {
  const double *obs_e;       /* n_obs (device) */
  const double *obs_n;
  const double *obs_u;
  int64_t n_obs;
  const double *prisms_soa;  /* 7 rows of prism_stride */
  int64_t prism_stride;
  int64_t n_prisms;
  int64_t chunk;             /* prisms per work item (multiple of 128) */
  int64_t n_chunks;          /* ceil(n_prisms / chunk) */
  double *partials;          /* n_chunks * n_obs doubles (device) */
  double *out;               /* n_obs doubles (device), harmonica units */
  int32_t *singular_flag;    /* device int32 or NULL */
  int32_t field;             /* field code 0..9 */
  int32_t check_singular;
} hg_problem_plan;

typedef struct hg_work_item {
  int32_t problem;  /* index into the problem table */
  int32_t tile;     /* 128-point tile */
  int32_t chunk;    /* prism chunk */
  int32_t pad;
} hg_work_item;

/*
 * Run one round: the items (device array) are grouped by field, in field-code
 * order, with field_counts[f] (host array of 10) items of field f; every
 * field present gets its own persistent launch over the problem table
 * (device array) with n_ctas CTAs (<= 0: one full wave of that field's
 * kernel); the potential gets two (its edge-log terms, then its face terms
 * added to the same partial sums).  `counter` is 80 bytes of device memory
 * (one counter per field) the call zeroes and uses.
 */
int hg_round_run(const hg_problem_plan *problems, const hg_work_item *items,
                 const int64_t *field_counts, int32_t n_ctas, void *counter, void *stream);

/* out = units * sum over chunks of partials, for the listed problems (device int32 ids). */
int hg_round_reduce(const hg_problem_plan *problems, const int32_t *problem_ids, int64_t n_ids,
                    void *stream);

/*
 * ---------------------------------------------------------------------------
 * Adjoint of the forward (new: the reference has no derivatives; it
 * replaces assembling a gradient from repeated prism_gravity calls,
 * gravity.py:51-236).  With weights w_i = dL/dd_i for the outputs d_i of
 * field `field` (harmonica units):
 *   grad_density[j] = sum_i w_i dd_i/drho_j                 (any field)
 *   grad_bottom[j]  = sum_i w_i dd_i/dbottom_j              (g_z only)
 *   grad_top[j]     = sum_i w_i dd_i/dtop_j                 (g_z only)
 * Any of the three outputs may be NULL.  Null prisms (and, for the layer,
 * the prisms its forward skips) get zero gradients.  The workspace
 * (hg_*_adjoint_workspace bytes) is required.
 */
int hg_prism_adjoint_workspace(int64_t n_obs, int64_t n_prisms, size_t *bytes);

int hg_prism_adjoint(const double *obs_e, const double *obs_n, const double *obs_u,
                     const double *weights, int64_t n_obs, const double *prisms_soa,
                     int64_t prism_stride, int64_t n_prisms, int32_t field, double *grad_density,
                     double *grad_bottom, double *grad_top, void *workspace,
                     size_t workspace_bytes, void *stream);

int hg_layer_adjoint_workspace(int64_t n_obs, int64_t n_east, int64_t n_north, size_t *bytes);

/* Layer version: gradients are (n_north, n_east) row-major like the layer grids. */
int hg_layer_adjoint(const double *obs_e, const double *obs_n, const double *obs_u,
                     const double *weights, int64_t n_obs, const double *centre_e, int64_t n_east,
                     const double *centre_n, int64_t n_north, const double *bottom,
                     const double *top, const double *density, double thickness_threshold,
                     int32_t field, double *grad_density, double *grad_bottom, double *grad_top,
                     void *workspace, size_t workspace_bytes, void *stream);

/*
 * ---------------------------------------------------------------------------
 * Magnetic field of uniformly magnetized prisms.  Replaces the loops of
 * _jit_prism_magnetic_field / _jit_prism_magnetic_component
 * (src/harmonica/_forward/prisms/magnetic.py:275-400) behind prism_magnetic
 * (:28-136): b = mu0/(4 pi) T M with T the unit-density gradient-tensor
 * kernel, in nT.  Prisms with zero volume or zero magnetization are skipped
 * (magnetic.py:410-440).
 *   hg_pack_prisms_magnetic: (n, 6) [w, e, s, n, b, t] + 3 magnetization
 *     vectors (A/m) -> 9 rows of prism_stride (w, e, s, n, b, t, m_e, m_n, m_u)
 *   component: 0 b_e, 1 b_n, 2 b_u, 3 all three (out = 3 rows of n_obs)
 */
int hg_pack_prisms_magnetic(const double *prisms_aos, const double *mag_e, const double *mag_n,
                            const double *mag_u, int64_t n_prisms, double *soa,
                            int64_t prism_stride, void *stream);

int hg_prism_magnetic_workspace(int64_t n_obs, int64_t n_prisms, int32_t component,
                                size_t *bytes);

int hg_prism_magnetic(const double *obs_e, const double *obs_n, const double *obs_u,
                      int64_t n_obs, const double *prisms_soa, int64_t prism_stride,
                      int64_t n_prisms, int32_t component, double *out, void *workspace,
                      size_t workspace_bytes, void *stream);

/*
 * ---------------------------------------------------------------------------
 * Point masses.  Replaces the loops point_mass_cartesian / point_mass_spherical
 * (src/harmonica/_forward/point.py:357-450) behind point_gravity (:30-268).
 * spherical = 0: obs/pts are easting, northing, upward (m), any field code;
 * spherical = 1: longitude, latitude (degrees), radius (m), potential or g_z.
 * masses in kg; out in harmonica units (g_z downward, mGal, Eotvos).
 */
int hg_point_forward_workspace(int64_t n_obs, int64_t n_points, size_t *bytes);

int hg_point_forward(const double *obs_1, const double *obs_2, const double *obs_3,
                     int64_t n_obs, const double *pts_1, const double *pts_2,
                     const double *pts_3, const double *masses, int64_t n_points,
                     int32_t spherical, int32_t field, double *out, void *workspace,
                     size_t workspace_bytes, void *stream);

/*
 * ---------------------------------------------------------------------------
 * Magnetic dipoles.  Replaces the loops behind dipole_magnetic
 * (src/harmonica/_forward/dipole.py:23-130, 292-360): b = mu0/(4 pi)
 * (3 (m . r) r / |r|^5 - m / |r|^3), r = point - dipole, in nT.
 * Coordinates in m (easting, northing, upward), moments in A m^2.
 * component: 0 b_e, 1 b_n, 2 b_u, 3 all three (out: rows e, n, u of n_obs).
 */
int hg_dipole_workspace(int64_t n_obs, int64_t n_dipoles, int32_t component, size_t *bytes);

int hg_dipole_magnetic(const double *obs_e, const double *obs_n, const double *obs_u,
                       int64_t n_obs, const double *dip_e, const double *dip_n,
                       const double *dip_u, const double *m_e, const double *m_n,
                       const double *m_u, int64_t n_dipoles, int32_t component, double *out,
                       void *workspace, size_t workspace_bytes, void *stream);

/*
 * ---------------------------------------------------------------------------
 * Equivalent sources (point sources with the Green's function 1 / distance).
 * hg_eqs_jacobian replaces jacobian_numba_parallel/serial
 * (src/harmonica/_equivalent_sources/utils.py:54-74) with
 * greens_func_cartesian (cartesian.py:635-644) or greens_func_spherical
 * (spherical.py:413-424): jac is n_obs x n_points, row-major, on the device.
 * hg_eqs_predict replaces predict_numba_parallel/serial (utils.py:77-96):
 * out[i] = sum_j coefs[j] / distance(i, j); workspace from
 * hg_point_forward_workspace (NULL when it returns 0).  spherical = 0:
 * easting, northing, upward (m); 1: longitude, latitude (degrees), radius (m).
 */
int hg_eqs_jacobian(const double *obs_1, const double *obs_2, const double *obs_3, int64_t n_obs,
                    const double *pts_1, const double *pts_2, const double *pts_3,
                    int64_t n_points, int32_t spherical, double *jac, void *stream);

int hg_eqs_predict(const double *obs_1, const double *obs_2, const double *obs_3, int64_t n_obs,
                   const double *pts_1, const double *pts_2, const double *pts_3,
                   const double *coefs, int64_t n_points, int32_t spherical, double *out,
                   void *workspace, size_t workspace_bytes, void *stream);

/*
 * ---------------------------------------------------------------------------
 * Tesseroids (spherical prisms) of constant density.  Replaces
 * jit_tesseroid_gravity_parallel/serial (src/harmonica/_forward/
 * tesseroid_gravity.py:236-333) with the adaptive discretisation and
 * Gauss-Legendre quadrature of _tesseroid_utils.py:18-295, and the
 * null-tesseroid discard (_tesseroid_utils.py:503-538), behind
 * tesseroid_gravity (tesseroid_gravity.py:35-216).
 *
 * longitude, latitude (degrees), radius (m): n_obs computation points.
 * tesseroids: n_tesseroids rows of (west, east, south, north, bottom, top)
 * in degrees and metres, row-major, already made continuous in longitude
 * (west <= east, as _check_tesseroids leaves them); density in kg/m^3: one
 * value per tesseroid (density_per_node = 0), or (density_per_node = 1) two
 * per tesseroid, the density at its two radial Gauss-Legendre nodes -- a
 * density function evaluated at radius_p as
 * gauss_legendre_quadrature_variable_density does
 * (_tesseroid_variable_density.py:18-107); valid only without radial
 * discretization, where every small tesseroid keeps its root's radii.
 * field: 0 potential (J/kg) or 3 g_z (mGal, downward).
 * radial_discretization: nonzero splits along the radius too.
 * stack_size (<= 100) and max_discretizations: the reference's STACK_SIZE
 * and MAX_DISCRETIZATIONS (tesseroid_gravity.py:27-28); <= 0 gives 100 and
 * 100000.
 * glq_nodes, glq_weights: HOST arrays of 6 (longitude, latitude, radius x 2
 * nodes), the degree-2 Gauss-Legendre rule (numpy leggauss(2) in the
 * reference); NULL uses -+1/sqrt(3) and weights 1.
 * status: optional device int32 OR-ed with 1 when a pair overflows the
 * stack ("Stack Overflow") and 2 when a pair needs more than
 * max_discretizations small tesseroids ("Exceeded maximum discretizations"); the
 * output is then not the reference's (which raises OverflowError).
 * Stream-ordered; workspace from hg_tesseroid_forward_workspace (NULL: the
 * call allocates stream-ordered).
 */
int hg_tesseroid_forward_workspace(int64_t n_obs, int64_t n_tesseroids, size_t *bytes);

int hg_tesseroid_forward(const double *longitude, const double *latitude, const double *radius,
                         int64_t n_obs, const double *tesseroids, const double *density,
                         int32_t density_per_node, int64_t n_tesseroids, int32_t field,
                         int32_t radial_discretization,
                         int32_t stack_size, int64_t max_discretizations,
                         const double *glq_nodes, const double *glq_weights, double *out,
                         int32_t *status, void *workspace, size_t workspace_bytes,
                         void *stream);

/*
 * Points inside tesseroids (_check_points_outside_tesseroids,
 * _tesseroid_utils.py:446-468): counts the (point, tesseroid) pairs with the
 * point strictly inside the tesseroid (longitude compared in [0, 360) and
 * [-180, 180)) into the device int64 *n_conflicts and stores the first
 * `capacity` of them as (point, tesseroid) index pairs in the device array
 * conflicts (2 x capacity int64, unordered).
 */
int hg_tesseroid_inside(const double *longitude, const double *latitude, const double *radius,
                        int64_t n_obs, const double *tesseroids, int64_t n_tesseroids,
                        int64_t *conflicts, int64_t capacity, int64_t *n_conflicts,
                        void *stream);

#ifdef __cplusplus
}
#endif

#endif /* HARMONICA_GB300_H */
