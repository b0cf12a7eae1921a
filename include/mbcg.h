/*
 * mbcg.h -- C ABI of the GB300 moment-based colour-gradient lattice Boltzmann step
 * (D3Q19 / D3Q27), a drop-in for the reference solver's time-step path.
 *
 * Lattice convention (same as the reference, utilities/indexing.cuh:10-14 and
 * utilities/bounds.cuh:12-20): an NX x NY x NZ box whose outermost layer on every axis is
 * a ghost frame.  Fluid nodes are 1..N-2 on each axis; the node (x,y,z) of field f lives at
 * f[x + y*pitch + z*pitch*NY] (pitch = NX in the reference's dense layout).  Periodic axes
 * wrap over the N-2 fluid nodes (bounds.cuh:34-77).
 *
 * State: 11 SoA moment fields per node, in this order (memory.cuh:14-29):
 *   0 rhor, 1 rhob, 2 ux, 3 uy, 4 uz, 5 Pixx, 6 Pixy, 7 Piyy, 8 Piyz, 9 Pizz, 10 Pixz.
 * In the FP16/BF16 storage form the same 11 slots hold scaled deviations:
 *   0 (rho - rho_nominal(phi)) / rho_scale, 1 the colour complement
 *   c = sign(phi) (1 - |phi|) of phi = (rhor-rhob)/rho (+0 pure red, -0 pure blue),
 *   2..4 u / u_ref, 5..10 Pi / pi_scale.
 *
 * Every function returns 0 on success and a negative MBCG_E* code on failure; the text of
 * the last error of the calling thread is available from mbcg_last_error().  Nothing here
 * calls exit() (the reference's CUDA_CHECK does, utilities/cudaUtilities.cuh:9-19).
 * Streams are caller-provided; a case handle must be driven by one host thread at a time.
 */
#ifndef MBCG_H
#define MBCG_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *mbcg_stream_t; /* == cudaStream_t; NULL = legacy default stream */

/* ---- enumerations ------------------------------------------------------------------ */
#define MBCG_NFIELDS 11

/* per-axis boundary kind */
#define MBCG_BC_PERIODIC 0 /* wrap over the N-2 fluid nodes (bounds.cuh:34-77)                 */
#define MBCG_BC_INOUT    1 /* jet axis: inlet ghost at 0, outlet ghost at N-1 (lbm.cuh:79-151,
                              jet/boundary_conditions.cuh:16-109)                             */
#define MBCG_BC_WALL     2 /* no-slip walls on the ghost layers 0 and N-1 (halfway bounce-back)*/

/* outlet kind for the INOUT axis */
#define MBCG_OUTLET_CONVECTIVE   0 /* reference: jet/boundary_conditions.cuh:45-109            */
#define MBCG_OUTLET_ZERO_GRADIENT 1 /* ghost = copy of the last fluid layer                      */

/* moment storage precision */
#define MBCG_FP32 0
#define MBCG_FP16 1
#define MBCG_BF16 2

/* initial-condition functor */
#define MBCG_IC_JET    0 /* jet/jetIn.cuh:16-60        */
#define MBCG_IC_BUBBLE 1 /* bubble/bubbleIn.cuh:15-52  */
#define MBCG_IC_RTI    2 /* rti/rtiIn.cuh:18-119       */
#define MBCG_IC_NONE   3 /* leave the state as copied in */

/* error codes */
#define MBCG_OK            0
#define MBCG_E_INVALID    -1 /* bad parameter                        */
#define MBCG_E_CUDA       -2 /* a CUDA runtime / driver call failed    */
#define MBCG_E_NOMEM      -3 /* device allocation failed               */
#define MBCG_E_TIMEOUT    -4 /* a bounded device wait or a server wait gave up */
#define MBCG_E_UNSUPPORTED -5

/* ---- case parameters (runtime replacement of the reference's constants.cuh) --------- */
typedef struct mbcg_params {
    int32_t q;              /* 19 or 27 (constants.cuh:21-26, stencil_ct.cuh:419-425)     */
    int32_t nx, ny, nz;     /* lattice size including the ghost frame (constants.cuh:14-16)*/
    int32_t bc[3];          /* MBCG_BC_* for x, y, z; at most one non-periodic axis        */
    int32_t outlet;         /* MBCG_OUTLET_*                                               */
    int32_t precision;      /* MBCG_FP32 / MBCG_FP16 / MBCG_BF16                           */
    int32_t ic;             /* MBCG_IC_* used by mbcg_init                                 */
    double tau;             /* relaxation time; oms = 1 - 1/tau (constants.cuh:78-85)       */
    double sigma;           /* surface tension (constants.cuh:90)                          */
    double beta;            /* recolouring parameter (constants.cuh:91)                    */
    double rho_r0, rho_b0;  /* nominal phase densities (constants.cuh:72-73); a ratio != 1
                               switches on the phase-dependent rest-population equilibrium */
    double gravity[3];      /* body-force acceleration; force density = rho * g (Guo)      */
    /* jet case (constants.cuh:31-35, jet/jetIn.cuh, jet/boundary_conditions.cuh) */
    double jet_radius;
    double jet_velocity;
    double jet_center[2];   /* disc centre in the two non-jet axes, in axis order          */
    double jet_phase;       /* phi of the injected fluid: -1 = blue (reference), +1 = red  */
    double inlet_noise;     /* relative amplitude of the per-step uniform inlet noise      */
    uint64_t seed;          /* counter-based RNG seed for the inlet noise                  */
    /* bubble case (constants.cuh:38-41, bubble/bubbleIn.cuh) */
    double bubble_radius;
    double bubble_center[3];
    double bubble_width;    /* 0 = sharp mask (reference); > 0 = tanh profile width        */
    double bubble_phase;    /* phi inside the bubble: -1 = blue (reference), +1 = red      */
    /* Rayleigh-Taylor case (constants.cuh:44-50, rti/rtiIn.cuh); the interface normal is
       the wall axis (or y when no axis is a wall) */
    double rti_position;
    double rti_amplitude;
    double rti_width;
    double rti_phase_above; /* phi above the interface: -1 = blue (reference), +1 = red    */
    int32_t rti_mode[2];    /* modes along the two transverse axes, in axis order          */
    int32_t omega2_conservative; /* 0 (reference): below |F| = 1e-4 cos2rule is 0 but Omega2
                               still subtracts A|F|B_i/2, which does not sum to zero
                               (forces.cuh:80-83, collisionOperators.cuh:16-25); 1: Omega2 is
                               zero there, so colour masses are conserved exactly          */
    int32_t wait_test_cycles; /* testing only, 0 in normal use.  > 0: the first plane wait of
                               every step tile waits on a barrier that nothing completes, giving
                               up after this many SM clock cycles, so the bounded-wait path runs:
                               the tile drains its in-flight copies and exits, and mbcg_status
                               reports 1 (the step's results are then incomplete)            */
    /* FP16/BF16 storage scales */
    double rho_scale;       /* (rho - rho_nominal) / rho_scale is stored; default 0.01     */
    double u_ref;           /* u / u_ref is stored; default 0.05                           */
    double pi_scale;        /* Pi / pi_scale is stored; default u_ref^2                    */
    /* phase-dependent relaxation (forces.cuh:101-108, defined but unused by the reference):
       0 (reference) = one relaxation time tau for both phases; > 0 = tau is the red phase's and
       tau_b the blue phase's, blended per node as tau_interface does,
       tau_eff = (1 + psi)/2 tau + (1 - psi)/2 tau_b, which sets oms = 1 - 1/tau_eff and the
       Omega2 amplitude sigma / (4 cs^4 tau_eff) at that node                               */
    double tau_b;
} mbcg_params;

/* Fill *p with the reference's shipped constants (constants.cuh:9-93): D3Q27, 128^3 jet
 * along y, tau = 1, sigma = 0.1, beta = 0.9, jet radius 12, velocity 0.05, blue jet. */
void mbcg_params_default(mbcg_params *p);

/* ---- moment views ------------------------------------------------------------------ */
/* 11 device arrays of one state, reference field order; the replacement of the
 * reference's MomentsDevice (memory.cuh:14-29) with an explicit row pitch. */
typedef struct mbcg_moments {
    void *f[MBCG_NFIELDS];
    int64_t pitch;          /* elements between rows (>= nx)                               */
    int32_t precision;      /* MBCG_FP32 / MBCG_FP16 / MBCG_BF16                           */
    int32_t reserved;
} mbcg_moments;

typedef struct mbcg_diag {
    double mass_r, mass_b;  /* sum of rhor / rhob over fluid nodes                         */
    double momentum[3];     /* sum of rho*u over fluid nodes                               */
    double p_in, p_out;     /* mean pressure inside the bubble core / far field (bubble)   */
    double dp;              /* p_in - p_out (Laplace pressure jump)                        */
    int64_t nonfinite;      /* fluid nodes with a non-finite field or rho <= 0             */
    int64_t nodes;          /* fluid nodes reduced over                                    */
} mbcg_diag;

/* ---- case handle: library-owned state -------------------------------------------- */
typedef struct mbcg_case mbcg_case;

/* Validates *p, allocates the two moment states (A current, B next; memory.cuh:153-164)
 * with a padded row pitch, builds the TMA descriptors.  No kernel runs. */
int mbcg_create(const mbcg_params *p, mbcg_case **out);
int mbcg_destroy(mbcg_case *c);

/* Initial condition p->ic on state A, then the initial boundary pass (main.cu:25-26). */
int mbcg_init(mbcg_case *c, mbcg_stream_t s);

/* nsteps fused steps: RCS (lbm.cuh:20-262) + boundary functors (kernels.cu:102-114) +
 * swap (memory.cuh:200-203), all in one kernel launch per step. */
int mbcg_step(mbcg_case *c, int32_t nsteps, mbcg_stream_t s);

/* The reference's split form for drop-in parity: mbcg_rcs writes B from A without the
 * boundary pass (launch_RCS, launch.cuh:89-94); mbcg_bc applies the boundary functors on B
 * reading the old state A (launch_JetBoundaryConditions, launch.cuh:78-83); mbcg_swap
 * exchanges A and B (swap_moments, memory.cuh:200-203). */
int mbcg_rcs(mbcg_case *c, mbcg_stream_t s);
int mbcg_bc(mbcg_case *c, mbcg_stream_t s);
int mbcg_swap(mbcg_case *c);

/* Device views of the current (A) and next (B) states. */
int mbcg_fields(const mbcg_case *c, mbcg_moments *a, mbcg_moments *b);
int64_t mbcg_steps_done(const mbcg_case *c);

/* Copies between state A and 11 host FP32 arrays in the reference's dense layout
 * (pitch = nx, copy_out_D2H in memory.cuh:209-217).  FP16/BF16 states are converted. */
int mbcg_copy_out(mbcg_case *c, float *const host[MBCG_NFIELDS], mbcg_stream_t s);
int mbcg_copy_in(mbcg_case *c, const float *const host[MBCG_NFIELDS], mbcg_stream_t s);

/* Host-resident states through the case: for j = 0..count-1, exactly
 *   mbcg_copy_in(c, in[j]); mbcg_step(c, nsteps); mbcg_copy_out(c, out[j]);
 * (the same bits), with in[j] = in + j * MBCG_NFIELDS and out[j] likewise (dense FP32 arrays
 * in the reference's layout).  The transfers of consecutive states overlap: the result of
 * state j moves to the host while state j+1 moves in and is stepped, so the host link carries
 * both directions at once (the host arrays should be pinned for that).  Holds four dense FP32
 * state images on the device (two in, two out; one each where memory is short), allocated on
 * first use and kept with the case.  Returns when out[count-1] is written;
 * the case's state is then the last result.  (No counterpart in the reference, whose host loop
 * copies one state out at a time: copy_out_D2H, memory.cuh:209-217.) */
int mbcg_run_host(mbcg_case *c, int32_t count, const float *const *in, float *const *out, int32_t nsteps,
                  mbcg_stream_t s);

/* FP64 on-GPU conservation and Laplace-pressure diagnostics of state A (synchronous). */
int mbcg_diagnostics(mbcg_case *c, mbcg_diag *out, mbcg_stream_t s);

/* Reads and clears the device status word.  0: every bounded device wait completed.  1: a wait
 * for a staged plane gave up; the tile then drained its in-flight copies with a bounded wait and
 * exited, so the step's results are incomplete.  Should that drain have given up as well, copies
 * could still land in shared memory after the block exited, and the word cannot tell the two
 * cases apart: treat any non-zero status as a poisoned context (stop launching on it, report the
 * error, do not re-run the step). */
int mbcg_status(mbcg_case *c, int32_t *status);

/* The parameters the case was created with. */
int mbcg_case_params(const mbcg_case *c, mbcg_params *out);

/* ---- in-situ phase statistics (no counterpart in the reference) ---------------------- */
/* The "tracked" phase is the injected one for a jet (the sign of jet_phase), else red
 * (phi > 0).  FP64 sums over the fluid nodes of state A, computed on the GPU. */
typedef struct mbcg_phase_stats {
    double volume_tracked;      /* fluid nodes where the tracked phase dominates (its phi > 0)   */
    double volume_other;
    double interface_area;      /* sum of |grad phi| / 2 (central differences): the area of a
                                   diffuse interface of any profile, in lattice units^2          */
    int64_t interface_nodes;    /* 4 rho_r rho_b / rho^2 > 1e-4 (lbm.cuh:181)                    */
    double penetration;         /* inlet/outlet axis: largest distance from the inlet ghost layer
                                   of a node where the tracked phase dominates; -1 otherwise      */
    double centroid[3];         /* centroid of the tracked phase (fluid-node coordinates)        */
    /* MBCG_STATS_COMPONENTS only (else -1): regions of the tracked phase connected through
     * faces, periodic axes wrapped */
    int64_t components;
    int64_t largest_component;  /* nodes in the largest region                                  */
    int64_t detached;           /* regions not touching the first fluid layer of the inlet axis
                                   (all regions without one): droplets                          */
    int64_t detached_volume;    /* nodes in them                                                */
    int32_t status;             /* non-zero: a bounded device loop gave up (results incomplete) */
    int32_t reserved;
} mbcg_phase_stats;

#define MBCG_STATS_COMPONENTS 1 /* also label connected regions (temporary: 8 bytes per node) */

int mbcg_phase_statistics(mbcg_case *c, int32_t flags, mbcg_phase_stats *out, mbcg_stream_t s);
/* The same on caller-owned arrays (reference layout, any pitch >= nx). */
int mbcg_phase_statistics_moments(const mbcg_params *p, const mbcg_moments *a, int32_t flags,
                                  mbcg_phase_stats *out, mbcg_stream_t s);

/* ---- output: VTI images (io/vtiWriter.cuh:60-164) and checkpoints ---------------------- */
#define MBCG_VTI_ASCII 0   /* the reference's encoding: Float32 ASCII DataArrays, "%.8e " per value,
                              one x row per line (io/vtiWriter.cuh:60-85)                      */
#define MBCG_VTI_RAW   1   /* the same arrays as VTK appended raw binary (UInt64 size headers) */
/* field_mask: bit f selects field f (0 rhor ... 10 Pixz, as reference FP32 moments); 0 selects
 * the reference's five fields rhor, rhob, ux, uy, uz (io/vtiWriter.cuh:88-127). */
#define MBCG_VTI_REFERENCE_FIELDS 0x1Fu

/* Writes state A of the case over the full lattice (ghost frame included, as the reference
 * does) to path.  Synchronous (write_vti_step_device, io/vtiWriter.cuh:151-164). */
int mbcg_write_vti(mbcg_case *c, const char *path, uint32_t field_mask, int32_t format, mbcg_stream_t s);

/* Asynchronous VTI output (no counterpart in the reference, which stops the run to write).
 * mbcg_writer_snapshot enqueues on stream s a dense copy of state A into one of max_pending
 * device snapshot buffers and returns: steps enqueued on s afterwards may run at once.  The
 * device-to-host copy runs on the writer's own stream and the file is written by the writer's
 * thread, both overlapping later steps.  When every buffer holds a snapshot not yet on disk,
 * snapshot blocks until one is written.  Each snapshot buffer holds the selected fields in
 * device memory and in pinned host memory. */
typedef struct mbcg_writer mbcg_writer;
int mbcg_writer_create(int32_t max_pending, mbcg_writer **out);
int mbcg_writer_snapshot(mbcg_writer *w, mbcg_case *c, const char *path, uint32_t field_mask,
                         int32_t format, mbcg_stream_t s);
/* Waits until every snapshot is on disk; returns the first write error since the last flush. */
int mbcg_writer_flush(mbcg_writer *w);
int mbcg_writer_destroy(mbcg_writer *w); /* flushes first */

/* Checkpoint (no counterpart in the reference): a binary file with the case parameters, the step
 * count (the inlet-noise counter) and the 11 stored fields in their storage precision over the
 * full lattice, with an FNV-1a checksum.  A case restored by mbcg_checkpoint_load continues bit
 * for bit as the saved case would have.  save synchronises s. */
int mbcg_checkpoint_save(mbcg_case *c, const char *path, mbcg_stream_t s);
int mbcg_checkpoint_load(const char *path, mbcg_case **out);

/* ---- launch shape (no counterpart in the reference, whose block is the compile-time
 * 32x4x2 of compile.sh:34-36) --------------------------------------------------------- */
/* Step CTA shape: block_rows warps (8 or 16) of 32 lanes; zchunk destination planes per CTA
 * along z.  mbcg_create picks a shape from a wave-filling model, or the shape an earlier
 * mbcg_autotune measured for the same lattice, precision, sizes and boundary features. */
int mbcg_get_shape(const mbcg_case *c, int32_t *block_rows, int32_t *zchunk);
int mbcg_set_shape(mbcg_case *c, int32_t block_rows, int32_t zchunk);
/* Times `repeats` steps for each candidate shape (both block shapes, several z depths) on this
 * case, keeps the fastest and records it for later cases with the same key.  The timed steps
 * read the current state and write the other one: the current state is unchanged.
 * *best_ms (may be null) receives the time of one step with the chosen shape.  Synchronous. */
int mbcg_autotune(mbcg_case *c, int32_t repeats, double *best_ms, mbcg_stream_t s);

/* ---- raw entry points on caller-owned moment arrays -------------------------------- */
/* launch_RCS(A, B, cfg) (launch.cuh:89-94) on arrays laid out as in the reference
 * (any pitch >= nx).  step is the index of the state B will hold (inlet noise key). */
int mbcg_rcs_moments(const mbcg_params *p, const mbcg_moments *a, const mbcg_moments *b,
                     int64_t step, mbcg_stream_t s);
/* launch_JetBoundaryConditions(B, Aold, cfg) (launch.cuh:78-83). */
int mbcg_bc_moments(const mbcg_params *p, const mbcg_moments *b, const mbcg_moments *a_old,
                    int64_t step, mbcg_stream_t s);
/* launch_Init{Jet,StaticBubble,RTI}(A, cfg) (launch.cuh:14-72) for p->ic, followed by the
 * initial boundary pass for the jet (main.cu:25-26). */
int mbcg_init_moments(const mbcg_params *p, const mbcg_moments *a, mbcg_stream_t s);

/* FP64 diagnostics of caller-owned moment arrays (reference layout, any pitch >= nx) that
 * allocate no memory, host or device.  No counterpart in the reference: it is for callers that
 * cannot allocate where they need the numbers -- solver loops whose device memory is entirely
 * taken by resident states, programs whose framework allocator owns the GPU (a cudaMalloc can
 * synchronise the device or fail under memory pressure), or code holding only MomentsDevice-style
 * arrays and no case handle.  The partial sums live in one fixed array compiled into the library
 * (about 385 KB, held on every GPU that loads it until the process exits); lattices above
 * 134,217,728 fluid nodes are rejected with MBCG_E_UNSUPPORTED.  Every call looks up that
 * array's device address with the calling thread's device current (so a device reset does not
 * leave a stale address); the first call on a device also loads the library's device code
 * there, so make it before any stream capture.  All calls share the array: calls that overlap on the GPU race, so serialise them
 * (same stream, or synchronise between them).  Synchronous: returns once *out is filled. */
int mbcg_diagnostics_static(const mbcg_params *p, const mbcg_moments *a, mbcg_diag *out, mbcg_stream_t s);

/* ---- serving: continuous batching of many lattices on one GPU ------------------------
 * No counterpart in the reference (one lattice per process, main.cu:25-55).  A server owns a
 * device arena and a worker thread.  Requests (a case and a step count) queue on submit and are
 * admitted while a slot and arena space are free, in the order the policy gives (with backfill
 * a later request that fits may pass one that does not yet).  All resident lattices advance
 * together: one persistent batch-kernel launch per time step runs every live lattice's tiles
 * from one flat queue, and each batch composition (the set of live lattices) is captured once
 * as a CUDA graph of chunk_steps launches that is replayed until the composition changes.  A
 * lattice computes the same arithmetic alone or in any mix (its tiles never read another
 * lattice's data), so its result is identical, bit for bit, whatever else runs beside it. */
typedef struct mbcg_server mbcg_server;

typedef struct mbcg_server_config {
    int64_t arena_bytes;    /* device memory for resident states (0: 70% of the free memory)  */
    int32_t max_live;       /* lattices resident at once (0: 64; at most 64)                   */
    int32_t chunk_steps;    /* launches per graph replay, the admission granularity (0: 16)    */
    int32_t keep_results;   /* 1: finished states stay resident until fetched or released      */
    int32_t backfill;       /* 1: admit later requests that fit while an earlier one waits     */
    int32_t zchunk;         /* z depth of the tiles (0: the planner picks one per composition:
                               the depth whose greedy schedule of all live tiles on the SMs,
                               under the cost model, gives the shortest launch)                */
    int32_t calibrate;      /* 1: measure the cost model (time of one tile plane per kernel body
                               and lattice, fixed cost per tile) at start-up; 0: defaults      */
    int32_t policy;         /* MBCG_POLICY_*: admission order (default FIFO: highest throughput;
                               SJF: lower median time to completion)                          */
    int32_t fill_waves;     /* shortest job first admits while the live tiles (at 16 planes)
                               fill fewer than fill_waves waves of one CTA per SM (0: 4)      */
} mbcg_server_config;

#define MBCG_POLICY_FIFO 0  /* arrival order                                                   */
#define MBCG_POLICY_SJF  1  /* shortest estimated remaining time first, with aging: a request's
                               wait counts against its work at the server's throughput        */

#define MBCG_REQ_QUEUED  0
#define MBCG_REQ_RUNNING 1
#define MBCG_REQ_DONE    2
#define MBCG_REQ_FAILED  3

typedef struct mbcg_request_info {
    int64_t id;
    int32_t state;          /* MBCG_REQ_*                                                      */
    int32_t status;         /* the lattice's device status word at completion (0 = ok)         */
    int64_t steps;          /* steps requested                                                 */
    int64_t steps_done;
    double t_submit;        /* seconds since the server started: submitted,                   */
    double t_admit;         /* admitted (its initial condition enqueued),                      */
    double t_done;          /* final state and diagnostics complete on the GPU (-1 if not)     */
    uint64_t state_hash;    /* order-independent 64-bit hash of the final fluid-node state     */
    mbcg_diag diag;         /* FP64 diagnostics of the final state                             */
} mbcg_request_info;

typedef struct mbcg_server_stats {
    int64_t submitted, completed, failed, live, queued;
    int64_t node_updates;   /* fluid-node updates completed                                    */
    int64_t compositions;   /* distinct batch compositions (graph captures)                    */
    int64_t replays;        /* graph replays                                                   */
    int64_t arena_bytes, arena_peak_bytes;
    int32_t zchunk;         /* tile z depth the planner chose for the current composition      */
    int32_t reserved;
    double plane_ns[10];    /* cost model: ns per tile plane of each batch-kernel body, in the
                               order Q19 FP32/FP16/BF16, Q27 FP32/FP16/BF16 (every feature),
                               Q19 FP32/FP16, Q27 FP32/FP16 (fully periodic, unforced)          */
    double tile_overhead_planes; /* cost model: fixed cost of a tile, in planes                */
    double busy_s;          /* first admission to the last completion                          */
} mbcg_server_stats;

void mbcg_server_config_default(mbcg_server_config *cfg);
int mbcg_server_create(const mbcg_server_config *cfg, mbcg_server **out);
/* Stops admitting, finishes the work in flight, frees everything. */
int mbcg_server_destroy(mbcg_server *s);
/* Queues a request (thread-safe, does not block).  The case's ic selects its initial condition;
 * a lattice larger than the whole arena is rejected with MBCG_E_NOMEM. */
int mbcg_server_submit(mbcg_server *s, const mbcg_params *p, int64_t nsteps, int64_t *id);
int mbcg_server_poll(mbcg_server *s, int64_t id, mbcg_request_info *out);
/* Blocks until request id is done or failed, or timeout_s passes (MBCG_E_TIMEOUT). */
int mbcg_server_wait(mbcg_server *s, int64_t id, double timeout_s, mbcg_request_info *out);
/* Blocks until nothing is queued or running. */
int mbcg_server_drain(mbcg_server *s, double timeout_s);
/* keep_results: copies a finished state to 11 dense FP32 host arrays (as mbcg_copy_out) and
 * keeps it resident; mbcg_server_release frees it. */
int mbcg_server_fetch(mbcg_server *s, int64_t id, float *const host[MBCG_NFIELDS]);
int mbcg_server_release(mbcg_server *s, int64_t id);
int mbcg_server_get_stats(mbcg_server *s, mbcg_server_stats *out);

/* Active (fluid) node count used by the MLUPS definition, (nx-2)(ny-2)(nz-2)
 * (utilities/mlups_count.cuh:24-29). */
int64_t mbcg_active_nodes(const mbcg_params *p);

/* Number of kernel launches one mbcg_step(c, 1, s) issues. */
int32_t mbcg_launches_per_step(const mbcg_case *c);

const char *mbcg_last_error(void);
const char *mbcg_version(void);

#ifdef __cplusplus
}
#endif
#endif /* MBCG_H */
