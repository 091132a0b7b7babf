/* tmcore_gpu.h - C ABI of the GB300 (sm_103a) TRiSK shallow-water library.
 *
 * Drop-in for the integrator and operator boundary of TMCORE
 * (TMCORE-Project/TMCORE).  The Fortran host keeps the namelist, mesh / state
 * I/O, logging and test cases; it calls these entry points through
 * iso_c_binding (a Fortran module of bind(C) interfaces, one per entry
 * point, with the same argument order).  Every entry point returns
 * 0 on success or a negative TMC_E* code, never exits or aborts; the message
 * of the last failure is tmc_last_error(h).  A handle owns one CUDA stream;
 * calls on one handle must not overlap (one handle per host thread).
 *
 * Element order at this ABI is always the caller's (the mesh file's) order;
 * the space-filling-curve renumbering used on the device is internal.
 * The state and field arrays of the handle calls (tmc_set_initial,
 * tmc_set_state, tmc_get_state, tmc_get_vertex, tmc_set_tracers,
 * tmc_get_tracers, tmc_time_integrate, tmc_spatial_operators, tmc_op_*,
 * tmc_history_fields, tmc_reconstruct, tmc_adv_*) may be HOST or DEVICE
 * pointers: the copies take their direction from unified addressing.  The
 * mesh (tmc_create), diagnostics (tmc_get_diag*), network parameters and
 * datasets (tmc_mlp_*), closure features and coarse-graining arrays are
 * host arrays unless stated otherwise.
 */
#ifndef TMCORE_GPU_H
#define TMCORE_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TMC_OK 0
#define TMC_E_ARG (-1)      /* bad argument or configuration */
#define TMC_E_CUDA (-2)     /* CUDA runtime error (message in tmc_last_error) */
#define TMC_E_HEALTH (-3)   /* non-finite state (tmc_get_diag), or a tensor-core wait ran out (tmc_mlp_*, and for the
                               closure in the step: tmc_get_diag, tmc_get_diag_all, tmc_time_integrate) */
#define TMC_E_UNSUP (-4)    /* option combination not implemented on the device */
#define TMC_E_STATE (-5)    /* call out of order (e.g. step before set_state) */

#define TMC_FP64 0 /* FP64 state and arithmetic; per element bit-identical to the reference order */
#define TMC_FP32 1 /* FP32 edge/vertex state and stencil arithmetic; FP64 metrics, gd and sums */

/* The MPAS grid exactly as src/core/mesh_mod.F90:130-167 reads it: unit
 * sphere, int32 1-based connectivity, Fortran (k, n) column-major arrays
 * (maxEdges = 6 or more, maxEdges2, vertexDegree = 3).  The library performs
 * the derivations of mesh_mod.F90:169-224 itself (areaEdge, fVertex,
 * nSignEdge, tSignEdge, verticesOnVertex, radius scaling, totalArea) and
 * copies everything; the caller keeps ownership of its arrays. */
typedef struct tmc_mesh_desc {
  int32_t nCells, nEdges, nVertices, maxEdges, maxEdges2, vertexDegree;
  const int32_t *nEdgesOnCell, *nEdgesOnEdge;
  const int32_t *cellsOnCell, *edgesOnCell, *verticesOnCell; /* (maxEdges, nCells) */
  const int32_t *cellsOnEdge, *verticesOnEdge;               /* (2, nEdges) */
  const int32_t *edgesOnEdge;                                /* (maxEdges2, nEdges) */
  const int32_t *cellsOnVertex, *edgesOnVertex;              /* (vertexDegree, nVertices) */
  const double *xCell, *yCell, *zCell, *latCell;
  const double *xEdge, *yEdge, *zEdge;
  const double *xVertex, *yVertex, *zVertex, *latVertex;
  const double *dvEdge, *dcEdge, *areaCell, *areaTriangle;
  const double *kiteAreasOnVertex; /* (vertexDegree, nVertices) */
  const double *weightsOnEdge;     /* (maxEdges2, nEdges) */
  const double *lonCell, *lonVertex; /* radians; lonVertex is required by the adv model only */
} tmc_mesh_desc;

/* namelist &tmcore (src/core/params_mod.F90:35-55), const_mod constants,
 * plus device options. */
typedef struct tmc_params {
  double dt;
  int32_t time_scheme;            /* 1 CRK3, 2 CRK4, 3 PC2 (time_scheme_mod.F90:47-184) */
  int32_t pv_scheme;              /* 1 APVM, 2 conservative APVM, 3 high-order upwind */
  int32_t conserve_energy;        /* energy-conserving beta (time_scheme_mod.F90:94-100,144-150,174-180) */
  int32_t flux_4th_order_correct; /* E-gradient correction with deriv3OnCell (tmcore_swm_mod.F90:183-195) */
  double apvm_weight;
  int32_t adv_order;              /* 2..6, upwind correction of gd on edges */
  int32_t adv_mono;
  int32_t interp_pv_order;        /* 3..6 for pv_scheme 3 */
  double radius, g, omega;        /* const_mod.F90:11-13 */
  int32_t n_tracers;              /* coupled mass-weighted tracers gd*q */
  int32_t tracer_adv_order;       /* 0: adv_order */
  int32_t tracer_adv_mono;
  int32_t precision;              /* TMC_FP64 or TMC_FP32 */
  int32_t renumber;               /* element order on the device: 0 as given, 1 Hilbert curve, 2 Morton curve */
  int32_t use_graph;              /* 1: one CUDA graph per RK step */
  int32_t diag_every;             /* invariants of the state every k steps (0: only on request) */
  int32_t device;                 /* CUDA device ordinal */
  int32_t block_size;             /* threads per block, 0 = tuned default */
  int32_t stencils;               /* 1: always build the poly-fit stencil tables (else only when used) */
  int32_t adv_wind;               /* 0: shallow-water model; adv model (tmcore_adv_mod.F90) with the
                                     prescribed wind 1 cosine-bell rotation, 2 deformation flow case 4 */
  int32_t members;                /* ensemble members sharing the mesh (FP32 shallow water, CRK4); 0 or 1: one */
  int32_t member_layout;          /* ensembles: 0 member-outermost arrays (every option), 1 member-innermost
                                     (members a multiple of 16; pv_scheme 1 with apvm_weight 0, or pv_scheme 3
                                     with interp_pv_order 3 or 4; adv_order 2, no tracers; other options:
                                     TMC_E_UNSUP): whole-line neighbour gathers */
  int32_t member_lanes;           /* member_layout 1: lanes of a warp per element, 8, 16 or 32, dividing
                                     members; a lane takes two members when members is a multiple of twice
                                     that, else one.  0 = automatic: 32 lanes (16 when members is not a
                                     multiple of 32), two members per lane when members is a multiple of 64 */
  int32_t reserved[2];
} tmc_params;

typedef struct tmc_handle tmc_handle;

/* Fill *p with the shipped SWM namelist (run/namelist.tmcore_swm) defaults. */
int tmc_default_params(tmc_params* p);

/* Replaces mesh_init + poly_fit_init + state/tend allocation
 * (src/core/tmcore_swm_mod.F90:29-47): copies and renumbers the mesh, builds
 * the stencil tables and allocates device state. */
int tmc_create(const tmc_mesh_desc* mesh, const tmc_params* params, tmc_handle** out);
int tmc_destroy(tmc_handle* h);
const char* tmc_last_error(const tmc_handle* h);

/* Initial condition: state(old)%cell%gd, state(old)%edge%u and
 * static%cell%ghs; runs the pre-loop of tmcore_swm_run
 * (tmcore_swm_mod.F90:62-71): gd_edge, iap_u = sqrt(gd_edge) u, invariants. */
int tmc_set_initial(tmc_handle* h, const double* gd, const double* u, const double* ghs);
/* Prognostic state(old) (gd on cells, iap_u on edges). */
int tmc_set_state(tmc_handle* h, const double* gd, const double* iap_u);
int tmc_get_state(tmc_handle* h, double* gd, double* iap_u, double* u);
/* Diagnostic pv and vorticity on vertices of state(old). */
int tmc_get_vertex(tmc_handle* h, double* pv, double* vor);
/* Coupled tracers, mass weighted gd*q, [n_tracers][nCells]. */
int tmc_set_tracers(tmc_handle* h, const double* qgd);
int tmc_get_tracers(tmc_handle* h, double* qgd);

/* nsteps iterations of tmcore_swm_run's loop body (tmcore_swm_mod.F90:75-88):
 * time_integrate (time_scheme_mod.F90:47-63) + time_advance; state stays on
 * the device.  Asynchronous unless an error is detected at launch. */
int tmc_step(tmc_handle* h, int32_t nsteps);
/* {total_mass, total_energy, total_potential_enstrophy,
 *  total_absolute_vorticity, beta} of state(old) (tmcore_swm_mod.F90:215-255,
 *  diag_mod.F90:76-91); synchronises.  Returns TMC_E_HEALTH (outputs filled)
 *  when an invariant is not finite: the state has left the physical range. */
int tmc_get_diag(tmc_handle* h, double out[5]);
/* the same for every ensemble member: out[members][5]; returns TMC_OK with
 * non-finite rows for members that blew up, so that a host can switch them
 * off or roll them back while the others continue */
int tmc_get_diag_all(tmc_handle* h, double* out);
int tmc_synchronize(tmc_handle* h);

/* time_integrate with host arrays: state(old) in, state(new) out, one step
 * (the whole drop-in for time_integrate at tmcore_swm_mod.F90:76).  qgd_old /
 * qgd_new are the coupled tracers ([n_tracers][nCells]) or NULL when
 * n_tracers = 0.  Page-locked host arrays give the fastest copies. */
int tmc_time_integrate(tmc_handle* h, const double* gd_old, const double* iap_u_old, const double* qgd_old,
                       double* gd_new, double* iap_u_new, double* qgd_new);

/* One call of spatial_operators (tmcore_swm_mod.F90:92-125). */
int tmc_spatial_operators(tmc_handle* h, const double* gd, const double* iap_u, double* tend_gd,
                          double* tend_iap_u);

/* Autotuner: times `steps` eager steps of the current state for each block
 * size in {64, 128, 192, 256, 384, 512} (256 at most for ensembles), one pass
 * of the fused step at a time (edge_flux, cell, vertex, edge_pv, final), keeps
 * the fastest per pass, restores the state and re-captures the step graphs.
 * block_sizes (may be NULL) receives {cell, vertex, edge_pv, edge_flux, final}. */
int tmc_autotune(tmc_handle* h, int32_t steps, int32_t block_sizes[5]);
/* Mean device time of one launch of each pass of the fused step over
 * `steps` eager steps (CUDA events around the pass; the steps advance the
 * state): ms = {cell, vertex, edge_pv (with the closure and conservative APVM
 * kernels), edge_flux, final update}. */
int tmc_pass_times(tmc_handle* h, int32_t steps, double ms[5]);

/* History diagnostics on the device (history_mod.F90:124-174 with
 * mpas_reconstruct, tmcore_swm_mod.F90:78-86): for state(old) of the selected
 * member, u on edges, the zonal and meridional wind on cells
 * (mpas_reconstruct_1d, mpas_vector_reconstruction.F90:207-261), h = (gd +
 * ghs)/g, div = div_operator(u) on cells, pv and vorticity on vertices.  Any
 * output pointer may be NULL.  The wind needs lonCell, latCell and
 * x/y/zEdge in tmc_mesh_desc.  tmc_reconstruct applies mpas_reconstruct_1d
 * to a given edge field (uX, uY, uZ: Cartesian components). */
int tmc_history_fields(tmc_handle* h, double* u, double* zonal, double* meridional, double* h_cell, double* div,
                       double* pv, double* vor);
int tmc_reconstruct(tmc_handle* h, const double* u, double* uX, double* uY, double* uZ, double* zonal,
                    double* meridional);

/* Ensembles (tmc_params.members > 1): every member is an independent model on
 * the same mesh, with its own state, topography, beta and invariants; the
 * members' arrays lie one after another and each kernel launch covers all of
 * them.  tmc_set_initial, tmc_set_state, tmc_get_state, tmc_get_vertex,
 * tmc_set_tracers, tmc_get_tracers and tmc_get_diag address the selected
 * member (initially 0); tmc_step advances all members.  tmc_time_integrate and
 * tmc_spatial_operators need members <= 1. */
int tmc_select_member(tmc_handle* h, int32_t member);

/* The learned PV-on-edge closure network: 24 -> 64 -> 64 -> 64 -> 1 with
 * GELU (tanh form) between hidden layers; TMC_MLP_PARAMS FP32 master
 * parameters in the order W1[64][24], b1[64], W2[64][64], b2[64],
 * W3[64][64], b3[64], W4[64], b4, used as BF16 weights (FP32 biases) with
 * FP32 accumulation.  Inputs are normalised as (x - x_mean) * x_inv_std and
 * the output is scaled by y_scale.  tmc_mlp_forward runs on the tensor cores
 * (tensor_cores = 1) or the CUDA cores (0); training is Adam (lr, beta1 0.9,
 * beta2 0.999, eps 1e-8) on the mean squared error over consecutive batches
 * of the stored dataset.  Arrays are host pointers. */
#define TMC_MLP_PARAMS 9985
#define TMC_MLP_FEATURES 24
typedef struct tmc_mlp tmc_mlp;
int tmc_mlp_create(int32_t device, uint64_t seed, tmc_mlp** out);
int tmc_mlp_destroy(tmc_mlp* n);
const char* tmc_mlp_last_error(const tmc_mlp* n);
int tmc_mlp_get_params(tmc_mlp* n, float* params);
int tmc_mlp_set_params(tmc_mlp* n, const float* params);
int tmc_mlp_set_scaling(tmc_mlp* n, const float* x_mean, const float* x_inv_std, float y_scale);
int tmc_mlp_forward(tmc_mlp* n, const float* x, int64_t rows, float* y, int32_t tensor_cores);
int tmc_mlp_set_dataset(tmc_mlp* n, const float* x, const float* y, int64_t rows);
int tmc_mlp_train(tmc_mlp* n, int32_t batch, int32_t steps, float lr, float* losses);
/* gradient of the mean squared error over rows (a multiple of 128) w.r.t.
 * the parameters, without updating them */
int tmc_mlp_gradient(tmc_mlp* n, const float* x, const float* y, int64_t rows, float* grad, double* loss);
/* Where tmc_mlp_train and tmc_mlp_gradient run: 1 (the default) the tensor
 * cores, forward and backward as tcgen05 MMAs of BF16 operands (weights,
 * activations and their gradients) with FP32 accumulation, the gradient
 * summed over blocks in a fixed order; 0 the CUDA cores, forward and
 * backward in FP32 from the BF16 weights.  TMC_E_HEALTH: a completion wait of
 * the tensor-core trainer timed out. */
int tmc_mlp_set_train_mode(tmc_mlp* n, int32_t tensor_cores);
/* No counterpart in the reference.  The output head: how the raw network
 * output y of an edge becomes the correction added to pv_edge, and what the
 * training loss fits (the mean of (correction - target)^2 / y_scale^2).
 *   head 0 (the default): y * y_scale, unconstrained.
 *   head 1: -softplus(y) dt (v (q_v2 - q_v1)/dvEdge + u (q_c2 - q_c1)/dcEdge),
 *     the APVM correction of operators_mod.F90:296-316 with a learned
 *     non-negative per-edge weight softplus(y) in place of apvm_weight; the
 *     direction comes from the edge's raw features (1, 22, 0, 23), dt is the
 *     model time step (> 0).  The correction keeps APVM's sign, so it can only
 *     remove potential enstrophy as APVM does.
 *   head 2: y * y_scale on the edges where y v (q_v2 - q_v1) <= 0 (APVM's
 *     sign along the edge: the correction removes potential enstrophy
 *     through q.F_perp there), 0 elsewhere; dt is not used.
 * Inside the energy-conserving q.F_perp form no head changes mass or energy. */
int tmc_mlp_set_head(tmc_mlp* n, int32_t head, double dt);
/* No counterpart in the reference (its errors abort, time_scheme_mod.F90:60).
 * Poll limit of the tensor-core kernels' completion waits (mbarrier polls
 * per MMA step; < 0 restores the default, 2^20).  A wait that runs out makes
 * the kernel flag TMC_E_HEALTH, wait with the default limit for the MMAs it
 * issued, free its tensor memory and return.  With 0 every such wait runs
 * out at once: this exercises that error path without withholding any
 * completion.  It applies to tmc_mlp_forward / train / gradient at once and
 * to a handle's closure from its next tmc_set_closure. */
int tmc_mlp_set_wait_limit(tmc_mlp* n, int32_t polls);

/* The learned closure in the FP32 CRK4 step: after the pv-on-edge pass of
 * every stage, the network's output for each edge (features: the stage's
 * u, tangential velocity, gd_edge, pv_edge, pv and gd on the two vertices /
 * cells, E, ghs and f on them, dvEdge, dcEdge, u on four neighbour edges, the
 * two pv gradients) is added to pv_edge before q.F_perp.  net = NULL turns it
 * off; the network must outlive its use.  tmc_set_member_closure switches it
 * per ensemble member (the invariant-drift fallback).  If a tensor-core
 * completion wait of the network runs out (a bounded wait; the tile group
 * that saw it leaves its remaining edges uncorrected and the step goes on),
 * the next tmc_get_diag, tmc_get_diag_all or tmc_time_integrate returns
 * TMC_E_HEALTH with its outputs filled; tmc_closure_status reports it as
 * *timed_out = 1.  Each of these reads and clears the flag, so one timeout is
 * reported once.  tmc_closure_features returns the
 * [nEdges][TMC_MLP_FEATURES] features and pv_edge of state(old) of the
 * selected member (caller's edge order), for training. */
int tmc_set_closure(tmc_handle* h, const tmc_mlp* net);
/* every_stage 1 (the default): the network runs on every stage's pv_edge;
 * 0: it runs in stage 1 and its output is held and added in stages 2-4. */
int tmc_set_closure_stages(tmc_handle* h, int32_t every_stage);
int tmc_set_member_closure(tmc_handle* h, int32_t member, int32_t on);
int tmc_closure_status(tmc_handle* h, int32_t* timed_out);
int tmc_closure_features(tmc_handle* h, float* features, double* pv_edge);
/* No counterpart in the reference.  The correction the network added to
 * pv_edge in stage 1 of the last step, for the selected member, [nEdges] in
 * the caller's edge order; needs the closure held from stage 1
 * (tmc_set_closure_stages(h, 0)) and a step taken with it.  With the state
 * the step started from, it is the network applied to that state's
 * tmc_closure_features. */
int tmc_closure_correction(tmc_handle* h, float* dq);

/* Coarse-graining of a fine-mesh state onto a coarser mesh (the closure's
 * training data and held-out truth).  Cells: kite-area-weighted means (each
 * fine kite goes to the coarse generator nearest its centre point; kites in
 * a tie band of 0.1 fine dcEdge between two generators are split equally).
 * Edges: the mean, over the fine edges within 0.75 fine dcEdge of the coarse
 * Voronoi edge and between its vertices, of the fine velocity u n + v t (v
 * the TRiSK tangential velocity) along the coarse normal; edge scalars (pv
 * on edges) are plain means over the same fine edges.  Host arrays in both
 * meshes' own order; any output pointer may be NULL.  device < 0 builds the
 * maps only (no CUDA; tmc_coarsen_apply then returns TMC_E_UNSUP).
 * tmc_coarsen_rows returns map `which` (0 cells, 1 normal velocity, 2 edge
 * scalars) as CSR rows over the fine array (start has a row count + 1
 * entries; NULL pointers return nnz only).  tmc_coarsen_unmatched counts
 * coarse edges without fine edges (their outputs are 0). */
typedef struct tmc_coarsen tmc_coarsen;
int tmc_coarsen_create(const tmc_mesh_desc* fine, const tmc_mesh_desc* coarse, int32_t device, tmc_coarsen** out);
int tmc_coarsen_apply(tmc_coarsen* c, const double* fine_gd, const double* fine_u, const double* fine_pv_edge,
                      double* coarse_gd, double* coarse_u, double* coarse_pv_edge);
int tmc_coarsen_rows(const tmc_coarsen* c, int32_t which, int64_t* nnz, int32_t* start, int32_t* idx, double* w);
int tmc_coarsen_unmatched(const tmc_coarsen* c, int64_t* edges);
/* the coarse cell (1-based) each fine cell is aggregated into */
int tmc_coarsen_cell_map(const tmc_coarsen* c, int32_t* coarse_cell_of_fine);
const char* tmc_coarsen_last_error(const tmc_coarsen* c);
int tmc_coarsen_destroy(tmc_coarsen* c);

/* MPAS grid files and history files in NetCDF classic format (CDF-1 and
 * 64-bit-offset CDF-2), read and written without the NetCDF library.
 * tmc_mesh_file_open reads the dimensions and arrays mesh_mod.F90:79-167
 * reads (the other variables are skipped) and fills *desc with pointers into
 * the file object, valid until tmc_mesh_file_close; arrays absent from the
 * file are NULL.  tmc_mesh_file_write writes the non-NULL arrays of a
 * tmc_mesh_desc as an MPAS grid file.  The history file holds the mesh
 * coordinates and, per tmc_history_write, one record of the fields of
 * history_mod.F90:124-174 (u, zonalWind, merdionalWind, h, pv, vor, div, tm,
 * te) of the handle's selected member at the given time. */
typedef struct tmc_mesh_file tmc_mesh_file;
int tmc_mesh_file_open(const char* path, tmc_mesh_file** out, tmc_mesh_desc* desc);
const char* tmc_mesh_file_error(const tmc_mesh_file* f);
int tmc_mesh_file_close(tmc_mesh_file* f);
int tmc_mesh_file_write(const char* path, const tmc_mesh_desc* desc);
typedef struct tmc_history tmc_history;
int tmc_history_create(const char* path, const tmc_mesh_desc* mesh, tmc_history** out);
int tmc_history_write(tmc_history* hw, tmc_handle* h, double seconds);
int tmc_history_close(tmc_history* hw);

/* Groups: several handles (different meshes and dt, each possibly an
 * ensemble) advanced together, e.g. a mixed batch of mesh levels with
 * dt = 1200 / 2^(level-4) s.  One CUDA graph per cycle of cycle_seconds holds
 * one independent branch per handle with cycle_seconds / dt steps (which must
 * be whole), so the handles' kernels run concurrently.  tmc_group_run is
 * asynchronous; later calls on a member handle are ordered after it.  The
 * handles must outlive the group and must not change their state size.  The
 * graph holds each handle's step as configured when the group was created
 * (closure, closure stages, block sizes): after changing those, create the
 * group again. */
typedef struct tmc_group tmc_group;
int tmc_group_create(tmc_handle* const* handles, int32_t n, double cycle_seconds, tmc_group** out);
/* The same with a choice of schedule (no counterpart in the serial
 * reference, which runs one model; state_mod.F90:88).  mode 0 is
 * tmc_group_create.  mode 1 advances the handles by one launch per pass over
 * all of them: every pass of a CRK4 stage is one kernel launch whose blocks
 * cover the element blocks of every handle that steps in that sub-step (the
 * handles ordered by steps per cycle, sub-step s of a cycle stepping those
 * with more than s steps), and the region sums, beta and the final update are
 * one launch each as well.  Mode 1 needs member-innermost ensembles
 * (member_layout 1) of one member count and one pv scheme, without the
 * learned closure, and at most 8 handles; otherwise it returns TMC_E_UNSUP
 * (with the reason in tmc_group_last_error of the returned group, which the
 * caller destroys).  The block sizes are those of the handle with the most
 * edges.  Members agree with mode 0 to FP32 rounding (the batch kernels run
 * the same per-block code, compiled into other kernels).  Mode 0 is the
 * faster schedule for a mixed batch whose largest level is latency bound:
 * its branches let the small levels use the bandwidth the large one leaves
 * idle, where mode 1 adds their work to every launch. */
int tmc_group_create_ex(tmc_handle* const* handles, int32_t n, double cycle_seconds, int32_t mode,
                        tmc_group** out);
int tmc_group_run(tmc_group* g, int32_t cycles);
int tmc_group_synchronize(tmc_group* g);
const char* tmc_group_last_error(const tmc_group* g);
int tmc_group_destroy(tmc_group* g);

/* The adv model (tmcore_adv_mod.F90, adv_wind = 1 or 2, FP64): one
 * advected scalar in place of gd, transported by the prescribed wind that
 * update_state re-sets at elapsed + the stage's dt (tmcore_adv_mod.F90:87-97);
 * tmc_step runs time_integrate with the adv spatial operator
 * (adv_scheme_sg11_mod.F90:33-48) and time_advance; tmc_get_diag gives the
 * total mass in out[0] (others 0).  tmc_adv_set_initial sets the scalar and
 * the wind at elapsed = 0 (test_cases_mod.F90:18-55). */
int tmc_adv_set_initial(tmc_handle* h, const double* q);
int tmc_adv_get(tmc_handle* h, double* q, double* u);
int tmc_adv_elapsed(tmc_handle* h, double* seconds);

/* Single operators of operators_mod.F90 (fine-grained parity, host arrays). */
int tmc_op_div(tmc_handle* h, const double* f_edge, double* div_cell);                 /* :40-55 */
int tmc_op_curl(tmc_handle* h, const double* f_edge, double* curl_vertex);             /* :76-91 */
int tmc_op_c2e(tmc_handle* h, const double* f_cell, double* f_edge);                   /* :93-104 */
int tmc_op_c2v(tmc_handle* h, const double* f_cell, double* f_vertex);                 /* :106-123 */
int tmc_op_v2c(tmc_handle* h, const double* f_vertex, double* f_cell);                 /* :125-141 */
int tmc_op_v2e(tmc_handle* h, const double* f_vertex, double* f_edge);                 /* :143-156 */
int tmc_op_kinetic_energy(tmc_handle* h, const double* u_edge, double* ke_cell);       /* :206-221 */
int tmc_op_tangent_wind(tmc_handle* h, const double* u_edge, double* v_edge);          /* :223-237 */
int tmc_op_tangent_vor_flux(tmc_handle* h, const double* u_edge, const double* gd_edge, /* :239-260 */
                            const double* pv_edge, double* out_edge);
int tmc_op_upwind_correction(tmc_handle* h, const double* f_cell, const double* u_edge, /* :423-472 */
                             double* f_edge_inout, int32_t order, int32_t mono);

/* Timing of the device path (CUDA events on the handle's stream).  If
 * ms_total is not NULL, nsteps steps run as tmc_step runs them (CUDA graph)
 * and *ms_total is their device time.  If ms_flux_kernel is not NULL, a
 * further nsteps steps run launch by launch with events around every edge
 * flux pass (the dominant kernel) and *ms_flux_kernel is the sum of those. */
int tmc_time_steps(tmc_handle* h, int32_t nsteps, double* ms_total, double* ms_flux_kernel,
                   int32_t* flux_launches, int32_t* total_launches);

/* Number of elements after load, and bytes of device memory held. */
int tmc_sizes(const tmc_handle* h, int64_t* nCells, int64_t* nEdges, int64_t* nVertices, int64_t* device_bytes);

/* Largest nCells / nEdges tmc_mass_energy_noalloc accepts. */
#define TMC_NOALLOC_MAX_ELEMENTS 8388608

/* No counterpart in the reference.  Total mass and total energy (the sums of
 * tmcore_swm_mod.F90:215-231, the values tmc_get_diag returns in out[0] and
 * out[1]) of a state held in DEVICE arrays, for callers that cannot call
 * cudaMalloc: a host that shares the GPU with a framework whose allocator
 * owns all device memory, or one whose policy forbids device allocations
 * while it runs.  It needs no handle and allocates nothing: its partial sums
 * live in a fixed 384 KiB array inside the library image, which every GPU
 * that loads the library keeps until the process exits.  Inputs: gd, ghs,
 * areaCell (m^2) for nCells cells and iap_u, areaEdge (m^2) for nEdges edges,
 * all device pointers, any element order.  Output: out[0] = mass,
 * out[1] = energy, a device pointer, written asynchronously on `stream`
 * (a cudaStream_t, NULL for the default stream).  Returns TMC_E_ARG when
 * nCells or nEdges is not in 1..TMC_NOALLOC_MAX_ELEMENTS.  The first call on
 * a device looks up the array's device address with that device current
 * and caches it; make that first call before any stream capture.  After
 * cudaDeviceReset of a device the cached address is stale: do not call it on
 * that device again in the same process.  Calls that overlap on the GPU
 * (other streams, other host threads on the same device) race on the shared
 * array. */
int tmc_mass_energy_noalloc(const double* gd, const double* ghs, const double* areaCell, int64_t nCells,
                            const double* iap_u, const double* areaEdge, int64_t nEdges, double* out, void* stream);

#ifdef __cplusplus
}
#endif
#endif
