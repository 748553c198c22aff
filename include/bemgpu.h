/*
 * bemgpu.h -- C ABI of libbemgpu.so, the GB300 (sm_103a) full-3D Helmholtz BEM library.
 *
 * The library replaces, for the dense full-3D boundary-element path of
 * AcousticScattering.jl, the reference's solve and its result queries:
 *
 *   bem(surface::Mesh, boundary, k; ...)         solvers/bem/surface.jl:10-23
 *   solve_full_bem(::Rigid|::PressureRelease)    solvers/bem/full.jl:52-184 (dense factor,
 *     or compression=(method=:hmatrix) + GMRES: bemgpu_hmatrix_solve)
 *   solve_full_bem(::FluidFilled)                solvers/bem/full.jl:273-495
 *   MixedRefinement (precision=:mixed)           solvers/bem/fluid_system.jl:172-309
 *   scattering_amplitude / far_field             solvers/bem/postprocessing.jl:1-13,
 *                                                solvers/bem/full.jl:509-519
 *   target_strength                              postprocessing/target_strength.jl:8,26
 *   pressure (full-BEM branch)                   fields/pressure.jl:404-471
 *   incidence_angle_sweep (full mesh)            postprocessing/sweeps.jl:626-701
 *   mesh(nodes, triangles) + topology checks     geometry/surface.jl:271-298, 341-405
 *
 * Discretisation: one unknown per flat triangle (centroid collocation), 7-point
 * degree-5 triangle rule for regular pairs, closed-form Laplace parts plus bounded
 * Helmholtz remainders for near pairs.  Kernel exp(ikr)/(4 pi r), exp(-i w t).
 *
 * Conventions shared with the reference:
 *   - nodes are 3 x N float64 column-major (one column per vertex), triangles 3 x M
 *     int64 column-major with 1-based vertex indices, (b-a)x(c-a) pointing outward;
 *   - incidence direction (cos b, sin b cos a, sin b sin a): polar angle b from +x,
 *     azimuth a from +y toward +z (solvers/bem/full.jl:14-18);
 *   - the default observation is backscatter, x_hat = -d (postprocessing.jl:4-6);
 *   - complex numbers are interleaved (re, im) float64 pairs.
 *
 * Every entry point returns a bemgpu_status; no entry point aborts the process.
 * Functions marked [host] run without a GPU.  Objects created from one context must
 * not be used from two host threads at the same time.
 */
#ifndef BEMGPU_H
#define BEMGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BEMGPU_API_VERSION 1

typedef enum {
  BEMGPU_OK = 0,
  BEMGPU_EINVAL = 1,        /* invalid argument (reference: ArgumentError) */
  BEMGPU_ETOPOLOGY = 2,     /* surface fails the closed/oriented/manifold checks */
  BEMGPU_ENOMEM_BUDGET = 3, /* request exceeds the context's HBM budget */
  BEMGPU_ESINGULAR = 4,     /* exact zero pivot in the double-precision factor */
  BEMGPU_ENOTCONVERGED = 5, /* refinement failed even after promotion */
  BEMGPU_ETIMEOUT = 6,      /* a bounded device wait gave up */
  BEMGPU_ECUDA = 7,         /* CUDA runtime error */
  BEMGPU_ENODEV = 8,        /* no usable CUDA device */
  BEMGPU_EBUSY = 9          /* request queue full */
} bemgpu_status;

typedef enum { BEMGPU_RIGID = 0, BEMGPU_PRESSURE_RELEASE = 1, BEMGPU_FLUID = 2 } bemgpu_boundary;

typedef enum {
  BEMGPU_FORMULATION_DEFAULT = -1, /* burton_miller (rigid/soft) or muller (fluid) */
  BEMGPU_BURTON_MILLER = 0,
  BEMGPU_CBIE = 1,
  BEMGPU_MULLER = 2
} bemgpu_formulation;

typedef enum { BEMGPU_DOUBLE = 0, BEMGPU_MIXED = 1 } bemgpu_precision;

/*
 * Precision of the regular (far) panel-pair quadrature.  Near and singular pairs, the
 * hypersingular term and every residual are always FP64.  DEFAULT means FP64 for
 * precision DOUBLE and FP32 for precision MIXED (the GB300 mixed pattern: every result
 * then states its error against the FP64 system); ASSEMBLY_DOUBLE with precision MIXED
 * reduces only the factorisation, which is the reference's precision=:mixed contract.
 */
typedef enum {
  BEMGPU_ASSEMBLY_DEFAULT = 0,
  BEMGPU_ASSEMBLY_DOUBLE = 1,
  BEMGPU_ASSEMBLY_SINGLE = 2
} bemgpu_assembly;

/* Refinement outcome, reference symbols of fluid_system.jl:186-307. */
typedef enum {
  BEMGPU_REASON_NONE = 0,
  BEMGPU_REASON_CONVERSION = 1,
  BEMGPU_REASON_SINGLE_SINGULAR = 2,
  BEMGPU_REASON_CONDITION = 3,
  BEMGPU_REASON_NONFINITE = 4,
  BEMGPU_REASON_ITERATION_LIMIT = 5,
  BEMGPU_REASON_STAGNATION = 6
} bemgpu_reason;

/* Field selector of pressure(); reference fields/pressure.jl:42-53. */
typedef enum {
  BEMGPU_FIELD_TOTAL = 0,
  BEMGPU_FIELD_SCATTERED = 1,
  BEMGPU_FIELD_INCIDENT = 2,
  BEMGPU_FIELD_INTERIOR = 3
} bemgpu_field;

/*
 * Discretisation of the rigid/soft equations.  COLLOCATION: constant panel values at the
 * centroids with analytic singular rules (this library's default).  NYSTROM: unknowns at
 * the seven quadrature nodes of every panel, kernel values times node weights, with a
 * density-interpolation correction of every node's own element, the discretisation of the
 * reference's solve_full_bem (full.jl:68-128 and 289-346 with correction=(method=:dim,));
 * one surface (rigid, pressure-release or fluid-filled), dense factor; pressure() leaves
 * the nearest element out of the node sum and recovers it by the same correction.
 */
typedef enum { BEMGPU_COLLOCATION = 0, BEMGPU_NYSTROM = 1 } bemgpu_discretization;

typedef struct bemgpu_ctx bemgpu_ctx;
typedef struct bemgpu_mesh bemgpu_mesh;
typedef struct bemgpu_factor bemgpu_factor;
typedef struct bemgpu_solution bemgpu_solution;

/*
 * One boundary-value problem on one surface.  Keyword arguments of the reference's
 * solve_full_bem (full.jl:52-58, 273-279) map to fields here.
 */
typedef struct {
  int32_t boundary;            /* bemgpu_boundary */
  int32_t formulation;         /* bemgpu_formulation */
  int32_t precision;           /* bemgpu_precision; mixed: complex64 factor + refinement */
  int32_t equilibrate;         /* row/column max scaling before the factor (default 1) */
  double k;                    /* exterior wavenumber [1/m], finite and > 0 */
  double density_contrast;     /* g = rho_int / rho_ext (fluid) */
  double soundspeed_contrast;  /* h = c_int / c_ext (fluid); k_int = k / h */
  double refine_tolerance;     /* backward-error acceptance (default 1e-13) */
  int32_t refine_maxiter;      /* corrections before promotion (default 8) */
  int32_t assembly;            /* bemgpu_assembly: precision of the regular-pair quadrature */
  double condition_guard;      /* single rcond guard (default 10 eps(float32)) */
  double near_eta;             /* near-pair radius in source diameters (default 2) */
  int32_t discretization;      /* bemgpu_discretization (default COLLOCATION) */
  int32_t condition_limit;     /* systems of at most this order get SVD condition numbers
                                  in their diagnostics (default 512, full.jl:364-409) */
  double norm_floor;           /* lower bound of the equilibration's row and column scales
                                  (default 0; precision DOUBLE only, as the reference) */
} bemgpu_problem;

/* Diagnostics of one solution; names follow the reference's diagnostics() fields. */
typedef struct {
  int64_t unknown_count;           /* n (rigid/soft) or 2n (fluid) */
  int64_t quadrature_nodes;        /* collocation points = panels */
  int64_t near_pairs;              /* pairs integrated with the singular rules */
  int32_t formulation;
  int32_t precision;               /* requested bemgpu_precision */
  int32_t factor_precision;        /* 0 single (complex64), 1 double (complex128) */
  int32_t refinement_reason;       /* bemgpu_reason (max severity over right-hand sides) */
  int32_t refinement_iterations;   /* corrections (max over right-hand sides) */
  int32_t equilibrate;
  double coupling_re, coupling_im; /* Burton-Miller alpha = i/k */
  double absolute_residual;        /* ||A x - b||_2 (max over right-hand sides) */
  double relative_residual;        /* ... / ||b||_2 */
  double scaled_absolute_residual; /* in the equilibrated equations */
  double scaled_relative_residual;
  double normwise_backward_error;
  double componentwise_backward_error;
  double single_reciprocal_condition; /* infinity-norm rcond of the complex64 factor */
  double assemble_ms, factor_ms, solve_ms, total_ms;
  int64_t device_bytes;            /* bytes held by the factor */
  int32_t nrhs;
  int32_t info;                    /* first exact zero pivot (1-based) of the factor, 0 if none */
  /* the reference's factor diagnostics (full.jl:364-409): 2-norm condition numbers of the
     system and of the equilibrated system from their singular values when the order is at
     most condition_limit (conditioning = 1, :svd), else conditioning = 0 (:not_computed)
     and both numbers NaN.  The factorisation keeps a copy of such a system; its SVDs run
     on the device when the diagnostics are first read. */
  double condition_number;
  double scaled_condition_number;
  int32_t conditioning;
  int32_t condition_limit;
  /* fluid Muller systems: how K' and H were evaluated, exterior and interior (the
     reference's derivative_evaluation, full.jl:201-212, 330-341): 1 direct quadrature;
     0 not used (rigid, soft, fluid CBIE) */
  int32_t derivative_exterior;
  int32_t derivative_interior;
} bemgpu_diagnostics;

/* ------------------------------------------------------------------ host utilities */
/* [host] Library version string. */
const char *bemgpu_version(void);
/* [host] Text of a status code. */
const char *bemgpu_status_string(int status);
/* [host] Fill a problem with the reference's defaults (rigid, Burton-Miller, double). */
void bemgpu_problem_init(bemgpu_problem *p);

/*
 * [host] Topology validation of a supplied flat-triangle surface, replacing
 * mesh(nodes, triangles) input checks (geometry/surface.jl:275-283) and
 * _validate_surface_topology (geometry/surface.jl:341-405): finite nodes, valid
 * indices, no repeated node, no degenerate triangle, exactly two triangles per edge
 * with opposite orientation, one connected component, manifold vertices, positive
 * enclosed volume.  resolution receives the longest edge.  BEMGPU_ETOPOLOGY or
 * BEMGPU_EINVAL with a message in err.
 */
int bemgpu_mesh_validate(const double *nodes, int64_t n_nodes, const int64_t *triangles,
                         int64_t n_triangles, double *resolution, char *err, size_t errlen);

/* [host] SHA-256 over (N, M, nodes, triangles) as little-endian int64/float64, hex. */
int bemgpu_mesh_hash(const double *nodes, int64_t n_nodes, const int64_t *triangles,
                     int64_t n_triangles, char out_hex[65]);

/*
 * [host] Near-pair list in CSR form: pair (i, j) is near when i == j or the squared
 * centroid distance is below eta^2 times the squared longest edge of panel j.
 * rowptr has n_triangles + 1 entries; *count receives the number of pairs; returns
 * BEMGPU_EINVAL (with *count set) when cap is too small.
 */
int bemgpu_near_pairs(const double *nodes, int64_t n_nodes, const int64_t *triangles,
                      int64_t n_triangles, double eta, int64_t *rowptr, int64_t *cols,
                      int64_t cap, int64_t *count);

/*
 * [host] Neighbourhoods of the restricted additive Schwarz preconditioner that
 * bemgpu_hmatrix_solve applies to Nyström rigid systems: for every triangle, the
 * min(count, n_triangles) triangles nearest to it (distances between the centroid nodes of
 * the 7-point rule, ties by index), itself first; out receives n_triangles x that many
 * 0-based indices.  No reference counterpart (the reference's rigid GMRES is
 * unpreconditioned).
 */
int bemgpu_schwarz_neighbourhoods(const double *nodes, int64_t n_nodes, const int64_t *triangles,
                                  int64_t n_triangles, int32_t count, int32_t *out);

/* ------------------------------------------------------------------ context */
/* Create a context on a device; hbm_budget_bytes = 0 means 90% of free memory. */
int bemgpu_ctx_create(int device, uint64_t hbm_budget_bytes, bemgpu_ctx **ctx);
int bemgpu_ctx_destroy(bemgpu_ctx *ctx);
/* Last error message of the context (or of the process when ctx is NULL). */
int bemgpu_last_error(const bemgpu_ctx *ctx, char *buf, size_t len);
/* Bytes currently held against the budget, and the budget. */
int bemgpu_ctx_memory(const bemgpu_ctx *ctx, uint64_t *used, uint64_t *budget);
/* Block until all work of the context has finished. */
int bemgpu_ctx_synchronize(bemgpu_ctx *ctx);

/* ------------------------------------------------------------------ meshes */
/* Validate (as bemgpu_mesh_validate), hash and upload a surface; panel geometry is
 * derived on the device. */
int bemgpu_mesh_upload(bemgpu_ctx *ctx, const double *nodes, int64_t n_nodes,
                       const int64_t *triangles, int64_t n_triangles, bemgpu_mesh **mesh);
int bemgpu_mesh_info(const bemgpu_mesh *mesh, int64_t *n_panels, double *resolution,
                     char hash_hex[65]);
int bemgpu_mesh_destroy(bemgpu_mesh *mesh);

/* ------------------------------------------------------------------ factor and solve */
/*
 * Assemble and factor the system of one problem (the reference's
 * _assemble_full_boundary / _assemble_full_fluid followed by _factor_fluid_system or
 * MixedRefinement.factorize_refined).  The factor keeps the complex128 system for
 * residuals and can serve any number of incidence directions.
 */
int bemgpu_factor_create(bemgpu_ctx *ctx, const bemgpu_mesh *mesh,
                         const bemgpu_problem *problem, bemgpu_factor **factor);

/*
 * Batched assembly + factorisation of `count` problems in fused launches (one CUDA
 * graph over all instances; meshes may differ in size).  factors[i] receives the
 * factor of problems[i].
 */
int bemgpu_factor_create_batch(bemgpu_ctx *ctx, int32_t count,
                               const bemgpu_mesh *const *meshes,
                               const bemgpu_problem *problems, bemgpu_factor **factors);

/*
 * Solve for nrhs plane waves with incidence (polar, azimuth) pairs in `incidence`
 * (2 * nrhs doubles).  Replaces _solve_full_boundary (full.jl:130-184) and
 * _solve_full_fluid (full.jl:456-495), including mixed refinement.
 */
int bemgpu_factor_solve(bemgpu_factor *factor, int32_t nrhs, const double *incidence,
                        bemgpu_solution **solution);

/* Solve many (factor, incidence set) pairs with batched kernels. */
int bemgpu_factor_solve_batch(bemgpu_ctx *ctx, int32_t count, bemgpu_factor *const *factors,
                              const int32_t *nrhs, const double *const *incidence,
                              bemgpu_solution **solutions);

int bemgpu_factor_destroy(bemgpu_factor *factor);
int bemgpu_factor_diagnostics(const bemgpu_factor *factor, bemgpu_diagnostics *out);

/* factor_create + factor_solve + factor_destroy: the reference's bem(surface, ...). */
int bemgpu_solve(bemgpu_ctx *ctx, const bemgpu_mesh *mesh, const bemgpu_problem *problem,
                 int32_t nrhs, const double *incidence, bemgpu_solution **solution);

/*
 * Coupled fluid regions: the reference's bem(surfaces, materials, k; parents, ...)
 * (solvers/bem/regions.jl:132-253).  surfaces[i] (i = 0..count-1, count <= 16) encloses
 * region i + 1; parents[i] is the region outside it: 0 for the unbounded exterior or the
 * 1-based index of an earlier surface (a nested chain is {0, 1, 2, ...}).  density[i] and
 * soundspeed[i] are region i + 1's contrasts relative to the exterior.  The surfaces must
 * not intersect; their containment is checked against the parents (BEMGPU_EINVAL
 * otherwise).  `problem` supplies k, the formulation (DEFAULT/MULLER or CBIE), precision,
 * refinement, assembly and near_eta (each surface uploaded with it); its boundary and
 * contrast fields are ignored.  The plane wave lights the surfaces that border the
 * exterior.  The solution answers far_field / target_strength (summed over those
 * surfaces, solvers/bem/postprocessing.jl:15-31), traces (scattered traces there, zero
 * on inner surfaces), region_traces, diagnostics and pressure_region.  With
 * problem->discretization = BEMGPU_NYSTROM the unknowns sit on the quadrature nodes of
 * every surface (7 per panel) and each surface's own operators are corrected at the
 * wavenumbers of both regions it borders; such a solution answers everything but
 * pressure (BEMGPU_EINVAL).
 */
int bemgpu_region_solve(bemgpu_ctx *ctx, int32_t count, const bemgpu_mesh *const *surfaces,
                        const double *density, const double *soundspeed, const int32_t *parents,
                        const bemgpu_problem *problem, int32_t nrhs, const double *incidence,
                        bemgpu_solution **solution);
/*
 * Unknowns of a coupled-region solution for right-hand side `rhs`, every panel in surface
 * order (2 * n doubles each): p = total pressure, v = the flux unknown (the interior normal
 * derivative is density_i * v, the exterior one density_parent * v).
 */
int bemgpu_region_traces(const bemgpu_solution *sol, int32_t rhs, double *p, double *v);

/* ------------------------------------------------------------------ hierarchical matrices */
/*
 * Compressed operators and GMRES: the reference's default rigid/soft path,
 * solve_full_bem(...; compression=(method=:hmatrix, tol), gmres_kwargs=(reltol, restart,
 * maxiter)) (full.jl:52-58, 68-184).  Complex128 throughout.
 */
typedef struct {
  double tol;         /* cross-approximation tolerance (compression tol, default 1e-5) */
  double eta;         /* admissibility min(diam s, diam t) < eta dist(s, t) (default 3) */
  int32_t leaf_size;  /* panels per leaf cluster, 8..64 (default 64) */
  int32_t restart;    /* GMRES restart length, 1..500 (default 150) */
  double reltol;      /* GMRES: stop when the residual <= max(reltol |b|, abstol) (1e-4) */
  double abstol;      /* (default 0) */
  int32_t maxiter;    /* GMRES Arnoldi steps (default 1200) */
  int32_t neighbours; /* Nyström rigid systems: elements per neighbourhood of a restricted
                         additive Schwarz right preconditioner, 0 = none (default), 1..128;
                         no reference counterpart (the reference's rigid GMRES is
                         unpreconditioned).  48 cuts GMRES steps 8x on meshes up to about
                         1300 panels and stalls GMRES on finer ones (one-level method) */
} bemgpu_hmatrix_options;

typedef struct {
  int64_t lowrank_blocks;    /* admissible blocks kept compressed */
  int64_t dense_blocks;      /* full blocks (leaf pairs + densified admissible blocks) */
  int64_t densified_blocks;  /* admissible blocks whose cross approximation hit the rank cap */
  int64_t lowrank_entries;   /* complex entries of U and V, both operators */
  int64_t dense_entries;     /* complex entries of the full blocks, both operators */
  int32_t max_rank, depth, leaves, pad;
  double compression;        /* stored entries / (2 n^2) */
  int32_t gmres_iterations;  /* Arnoldi steps, max over right-hand sides */
  int32_t gmres_converged;   /* 1 when every right-hand side met the tolerance */
  double build_ms, gmres_ms;
} bemgpu_hmatrix_stats;

/* [host] Fill options with the reference's defaults. */
void bemgpu_hmatrix_options_init(bemgpu_hmatrix_options *opt);
/*
 * [host] Block partition of the compressed operators of a surface (no device work):
 * counts = {admissible blocks, full blocks, leaves, tree depth}; blocks (optional, room
 * for cap blocks of 5 int32: kind 0 full / 1 admissible, first row, rows, first column,
 * columns, in permuted positions); perm (optional, n_triangles int32: permuted position
 * -> panel).  near_eta as for bemgpu_near_pairs.
 */
int bemgpu_hmatrix_plan(const double *nodes, int64_t n_nodes, const int64_t *triangles,
                        int64_t n_triangles, double near_eta, const bemgpu_hmatrix_options *opt,
                        int64_t counts[4], int32_t *blocks, int64_t cap, int32_t *perm);
/*
 * Rigid / pressure-release solve with compressed operators and GMRES for nrhs plane waves
 * (incidence as for bemgpu_factor_solve).  The returned solution answers every query.
 * GMRES that stops without meeting the tolerance returns BEMGPU_OK with gmres_converged =
 * 0, as the reference warns and returns (full.jl:157-159).
 */
int bemgpu_hmatrix_solve(bemgpu_ctx *ctx, const bemgpu_mesh *mesh, const bemgpu_problem *problem,
                         const bemgpu_hmatrix_options *opt, int32_t nrhs,
                         const double *incidence, bemgpu_solution **solution);
/* Compression and GMRES statistics of a solution from bemgpu_hmatrix_solve. */
int bemgpu_hmatrix_stats_get(const bemgpu_solution *sol, bemgpu_hmatrix_stats *stats);
/*
 * GMRES residual estimates of right-hand side rhs, one per Arnoldi step (the reference's
 * residual_history); writes min(cap, steps) values and the step count.
 */
int bemgpu_gmres_history(const bemgpu_solution *sol, int32_t rhs, double *out, int32_t cap,
                         int32_t *count);

/* ------------------------------------------------------------------ queries */
/*
 * Far-field amplitude f(x_hat) of right-hand side `rhs` at ndir unit directions
 * (3 * ndir doubles); out receives 2 * ndir doubles.  dirs == NULL means backscatter.
 * Replaces far_field (full.jl:509-519) / scattering_amplitude (postprocessing.jl:1-13).
 */
int bemgpu_far_field(bemgpu_solution *sol, int32_t rhs, int64_t ndir, const double *dirs,
                     double *out);
/* 20 log10 |f| at the same directions (target_strength.jl:8, 26). */
int bemgpu_target_strength(bemgpu_solution *sol, int32_t rhs, int64_t ndir,
                           const double *dirs, double *out);
/* Scattered surface traces p_scat, dpdn_scat of one right-hand side (2 * n doubles each). */
int bemgpu_traces(const bemgpu_solution *sol, int32_t rhs, double *p_scat, double *dpdn_scat);
int bemgpu_solution_diagnostics(const bemgpu_solution *sol, bemgpu_diagnostics *out);
/*
 * Pressure at npts points (3 * npts doubles, out 2 * npts doubles) by the layer
 * potentials of the surface traces, fields/pressure.jl:404-471.  Points on the
 * surface or on the wrong side for `field` give BEMGPU_EINVAL.
 */
int bemgpu_pressure(bemgpu_solution *sol, int32_t rhs, int64_t npts, const double *points,
                    int32_t field, double *out);
/*
 * pressure(sol, points; field, region) of a coupled-region solution
 * (fields/regions.jl:30-65): region = -1 evaluates each point in the region that contains
 * it (on an interface: the outer region, or the inner one for the interior field);
 * region >= 0 selects a region the point belongs to.  The total field in the unbounded
 * region adds the incident wave; field=:scattered needs the unbounded region and
 * field=:interior a bounded one (BEMGPU_EINVAL otherwise, as the reference's ArgumentError).
 * bemgpu_pressure on a coupled-region solution is this call with region = -1.
 */
int bemgpu_pressure_region(bemgpu_solution *sol, int32_t rhs, int64_t npts,
                           const double *points, int32_t field, int32_t region, double *out);
int bemgpu_solution_destroy(bemgpu_solution *sol);

/* ------------------------------------------------------------------ serving */
/*
 * Request loop over one context.  A request is one surface and boundary problem at nfreq
 * wavenumbers and nangles incidence directions; each (request, wavenumber) is one work
 * item.  Continuous batching over `lanes` worker threads, each with its own CUDA streams,
 * so that several batches are on the device at once: whenever a lane is free it takes a
 * batch of one size class (items whose system order is within a factor of two of the
 * head item's; the head is the oldest waiting item, or the oldest of another class when
 * another lane already runs that class, so a small request overtakes a large one), at
 * most max_batch factorisations, within the HBM budget left by the other lanes' batches
 * and the cache; it factors the items whose (mesh, k, boundary, precision) factor is not
 * cached, solves all of them in one batched launch sequence and completes the requests
 * whose items are all done.  Requests that arrive while batches run are admitted as soon
 * as a lane and memory free up.  Factors stay cached (LRU, cache_bytes) for reuse by
 * later requests on the same mesh and wavenumber (sweeps.jl:680-701 reuses a factor
 * across angles within one call); a factor is computed once and used by one lane at a
 * time.  Every item is computed exactly as alone: batching changes which launch carries
 * it, not its arithmetic.  A batch whose device allocation runs out of memory (the budget
 * counts live blocks, not the caching pools' free ones) is re-run once, when no other
 * batch is on the device; a second failure fails its requests.
 */
typedef struct bemgpu_server bemgpu_server;

typedef struct {
  int32_t max_batch;     /* factorisations per batch (default 64) */
  int32_t queue_limit;   /* pending requests before submit returns BEMGPU_EBUSY (4096) */
  uint64_t cache_bytes;  /* bytes of cached factors kept between batches (default budget/4) */
  int32_t lanes;         /* batches on the device at once, each on its own streams (2; 1..8) */
  int32_t reserved;
} bemgpu_server_options;

typedef struct {
  int64_t submitted, completed, failed;
  int64_t items, factorizations, cache_hits, batches;
  int64_t evictions;
  double busy_ms;        /* device time of all batches */
  uint64_t cached_bytes;
  int64_t retries;       /* items re-run after their batch ran out of device memory (once
                            each, with no other batch on the device) */
} bemgpu_server_stats;

void bemgpu_server_options_init(bemgpu_server_options *o);
int bemgpu_server_create(bemgpu_ctx *ctx, const bemgpu_server_options *opts,
                         bemgpu_server **server);
/* ks: nfreq wavenumbers (problem->k is ignored); incidence: 2 * nangles (polar, azimuth). */
int bemgpu_server_submit(bemgpu_server *server, const bemgpu_mesh *mesh,
                         const bemgpu_problem *problem, int32_t nfreq, const double *ks,
                         int32_t nangles, const double *incidence, int64_t *ticket);
/* Wait up to timeout_ms (< 0: forever) for a request.  amplitudes receives the
 * backscatter amplitudes (2 * nfreq * nangles doubles, frequency-major), latency_ms the
 * time from submit to completion.  BEMGPU_ETIMEOUT if not done in time; the request's
 * own failure status otherwise.  A waited request is released. */
int bemgpu_server_wait(bemgpu_server *server, int64_t ticket, int32_t timeout_ms,
                       double *amplitudes, double *latency_ms);
int bemgpu_server_stats_get(bemgpu_server *server, bemgpu_server_stats *stats);
/* Stops the worker after the running batch; pending requests fail with BEMGPU_EBUSY. */
int bemgpu_server_destroy(bemgpu_server *server);

/* ------------------------------------------------------------------ dense linear algebra */
/*
 * Solve A X = B for a caller-supplied dense complex matrix (n x n column-major,
 * interleaved complex128) and nrhs right-hand sides (n x nrhs, overwritten by X), with
 * the same equilibrated factor / mixed refinement the BEM systems use.  Replaces
 * _factor_fluid_system + _solve_fluid_system (full.jl:364-440) for hand-built
 * matrices; diag (optional) receives the refinement report.
 */
int bemgpu_dense_solve(bemgpu_ctx *ctx, int64_t n, const double *A, int32_t nrhs, double *B,
                       int32_t precision, int32_t equilibrate, double refine_tolerance,
                       int32_t refine_maxiter, double condition_guard,
                       bemgpu_diagnostics *diag);

/* Assembled operators of a problem for inspection (rigid/soft: M1 and M2 n x n, or 7n x 7n
 * on the quadrature nodes for the Nyström discretisation, corrections applied; fluid: A
 * 2n x 2n in M1, M2 unused).  Column-major interleaved complex128. */
int bemgpu_assemble_dense(bemgpu_ctx *ctx, const bemgpu_mesh *mesh,
                          const bemgpu_problem *problem, double *M1, double *M2);

/*
 * Products Y = M X of the compressed rigid/soft operators (op 0: M1, op 1: M2 as in
 * bemgpu_assemble_dense) with nr columns (n x nr column-major interleaved complex128),
 * for inspecting the compression; stats (optional) receives the operators' statistics.
 */
int bemgpu_hmatrix_apply(bemgpu_ctx *ctx, const bemgpu_mesh *mesh, const bemgpu_problem *problem,
                         const bemgpu_hmatrix_options *opt, int32_t op, int32_t nr,
                         const double *X, double *Y, bemgpu_hmatrix_stats *stats);

/*
 * Launch-shape autotuner (default on): the first time a batch shape is met, the compact
 * residual's rows per thread are chosen by timing the candidates.  Every candidate
 * computes bit-identical results.  enable = 0 switches it off and forgets the measured
 * choices (fixed rules are used).  No reference counterpart.
 */
int bemgpu_ctx_set_autotune(bemgpu_ctx *ctx, int32_t enable);
/*
 * CUDA graphs of the batched LU (default 1): the launch sequence of the tensor-core
 * factorisation of a batch is captured the second time a batch of the same shape (the
 * instances' orders) is factored, and replayed for later batches of that shape, with the
 * new batch's descriptors written into the graph's arrays (16 shapes per context, least
 * recently used dropped; not while profiling is on, nor on server lanes).  Results are
 * bit-identical with graphs on or off.  enable = 0 drops the captured graphs.  No
 * reference counterpart.
 */
int bemgpu_ctx_set_graphs(bemgpu_ctx *ctx, int32_t enable);
/*
 * Test hook for the out-of-memory path: the next `count` device allocations of the
 * context and its lanes fail as if cudaMalloc had returned cudaErrorMemoryAllocation (the
 * driver is not called; 0 cancels).  No reference counterpart.
 */
int bemgpu_ctx_inject_alloc_failures(bemgpu_ctx *ctx, int32_t count);
/* Batched-LU graphs captured and replayed by the context so far. */
int bemgpu_ctx_graph_stats(const bemgpu_ctx *ctx, int64_t *captures, int64_t *replays);
/*
 * Complex64 trailing updates of the mixed-precision LU on the tensor cores (split-BF16
 * tcgen05 GEMM, default 1) or on the CUDA cores (0).  No reference counterpart: a
 * switch for the precision study and for tests.
 */
int bemgpu_ctx_set_tensor_lu(bemgpu_ctx *ctx, int32_t enable);

/*
 * C -= A B for complex64 column-major A (m x k), B (k x n), C (m x n) through the
 * tensor-core update used by the mixed-precision LU (testing hook).
 */
int bemgpu_debug_cgemm(bemgpu_ctx *ctx, int64_t m, int64_t n, int32_t k, const float *A,
                       const float *B, float *C);

/*
 * C -= A B for complex64 column-major device matrices A (m x k, leading dimension lda),
 * B (k x n, ldb) and C (m x n, ldc), on `stream` (a cudaStream_t; NULL = default
 * stream), through the same tensor-core update as the mixed-precision LU -- without
 * allocating any device memory.  No counterpart in the reference: it exists for callers
 * that cannot allocate device memory where they need this update, such as hosts whose
 * free HBM is owned by their own pool allocator and real-time codes that may not
 * allocate after start-up.  The operand images, descriptors and timeout word live in a
 * file-scope device array of 4 MiB + 2 KiB that every GPU loading the library holds
 * until the process exits; hence m, n <= 2048 and k <= 128 (larger sizes return
 * BEMGPU_EINVAL).  Every call looks up that array's address on the current device
 * (cudaGetSymbolAddress; the first call on a device may load the module there, so make
 * it before any stream capture); `stream` must belong to the current device
 * (BEMGPU_EINVAL otherwise).  All calls share the array: calls whose GPU work overlaps
 * race.  The call waits for its stream and returns BEMGPU_ETIMEOUT if a bounded wait
 * gave up.
 * Errors are reported through bemgpu_last_error(NULL, ...).
 */
int bemgpu_cgemm_update_noalloc(void *stream, int64_t m, int64_t n, int32_t k, const void *A,
                                int64_t lda, const void *B, int64_t ldb, void *C, int64_t ldc);

/* ------------------------------------------------------------------ profiling */
/*
 * Kernel timing with CUDA events recorded on the launching stream around every launch
 * of the named kernel family ("assemble", "near", "getf2", "trsm", "gemm", "gemm_tc",
 * "far_field", "residual", ...).  enable = 0 stops recording; read returns the number
 * of launches and their summed device time since the last reset.
 */
int bemgpu_profile_enable(bemgpu_ctx *ctx, int32_t enable);
int bemgpu_profile_reset(bemgpu_ctx *ctx);
int bemgpu_profile_read(bemgpu_ctx *ctx, const char *family, int64_t *launches,
                        double *total_ms);
/* Number of library kernel launches issued by the process so far. */
int bemgpu_launch_count(const bemgpu_ctx *ctx, int64_t *count);
/* Device timer on the context's stream: start records a CUDA event; stop records a
 * second one, waits for it and returns the elapsed device time in milliseconds. */
int bemgpu_timer_start(bemgpu_ctx *ctx);
int bemgpu_timer_stop(bemgpu_ctx *ctx, double *ms);

#ifdef __cplusplus
}
#endif
#endif /* BEMGPU_H */
