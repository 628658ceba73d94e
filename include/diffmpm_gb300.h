/*
 * diffmpm_gb300 -- C ABI of the GB300 (sm_103a) explicit MPM step.
 *
 * This library replaces the explicit time step of geoelements/diffmpm
 * (diffmpm/solver.py, scheme.py, mesh.py, element.py, particle.py,
 * material.py, constraint.py, forces.py, functions.py).  The reference has no
 * foreign-function interface: its step is composed by string method dispatch
 * (diffmpm/mesh.py:31-58) in the order of diffmpm/scheme.py:22-67.  Each entry
 * point below names the reference interface it stands in for.
 *
 * Conventions
 *   - Every function returns an MpmStatus (0 = success).  mpm_last_error()
 *     gives a message for the last failure on a handle.
 *   - Buffers are caller-owned.  `on_device` = 1 means the pointer is device
 *     memory on the handle's GPU; 0 means host memory (the copy is done and
 *     synchronised inside the call).  The handle owns all simulation state
 *     and scratch (particle and nodal arrays, sort buffers, snapshots).
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default
 *     stream).  Calls are stream-ordered; one handle per host thread.
 *   - Particle arrays use the reference's layouts flattened row-major:
 *     loc/velocity (n, ndim), stress/strain Voigt (n, 6) in the order
 *     [xx, yy, zz, xy, yz, xz], scalars (n).  Reads return the original
 *     particle order whatever the internal (cell-sorted) order is.
 *   - Arithmetic is float32 throughout, as the reference's JAX default.
 */
#ifndef DIFFMPM_GB300_H
#define DIFFMPM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPM_ABI_VERSION 1

typedef struct MpmHandle MpmHandle;

typedef enum MpmStatus {
    MPM_OK = 0,
    MPM_ERR_INVALID = 1,      /* bad argument, shape or value (reference: ValueError/KeyError) */
    MPM_ERR_CUDA = 2,         /* a CUDA runtime call failed */
    MPM_ERR_OUT_OF_MESH = 3,  /* a particle left the mesh (reference: silent wrap/clamp ids) */
    MPM_ERR_CFL = 4,          /* a particle crossed more than one cell in one step */
    MPM_ERR_UNSUPPORTED = 5,  /* configuration this build does not implement */
    MPM_ERR_STATE = 6,        /* call out of order (e.g. step before initialize) */
    MPM_ERR_NOMEM = 7         /* device allocation failed */
} MpmStatus;

typedef enum MpmMaterialType {
    MPM_LINEAR_ELASTIC = 0,   /* diffmpm/material.py:54-116 */
    MPM_SIMPLE = 1,           /* diffmpm/material.py:119-131 */
    MPM_NEWTONIAN = 2         /* build definition; no counterpart in the reference */
} MpmMaterialType;

typedef struct MpmMaterial {
    int type;                 /* MpmMaterialType */
    double density;
    double youngs_modulus;    /* LinearElastic */
    double poisson_ratio;     /* LinearElastic */
    double E;                 /* SimpleMaterial */
    double bulk_modulus;      /* Newtonian */
    double dynamic_viscosity; /* Newtonian */
} MpmMaterial;

typedef enum MpmScheme { MPM_USF = 0, MPM_USL = 1 } MpmScheme;

/* Simulation description: the arguments of Quadrilateral4Node / Linear1D
 * (diffmpm/element.py:358-412, 626-690), MPMExplicit (diffmpm/solver.py:24-80),
 * Constraint (diffmpm/constraint.py:7-20), NodalForce (diffmpm/forces.py:9-18),
 * Linear/Unit (diffmpm/functions.py:16-49) and the material classes. */
typedef struct MpmDesc {
    int ndim;                      /* 2 = Quadrilateral4Node, 1 = Linear1D */
    int nelements[2];              /* nx, ny */
    double el_len[2];              /* hx, hy (converted to float32 like jnp.asarray) */
    int scheme;                    /* MpmScheme */
    int velocity_update;           /* 0/1 (diffmpm/particle.py:235-245) */
    int reinit_each_step;          /* 1: solve_jit semantics (volume/mass reset each step,
                                      diffmpm/solver.py:81-85,100-111); 0: solve semantics */
    double dt;
    double gravity[2];
    /* velocity constraints, flattened (node, dir, velocity), applied in order */
    int n_constraints;
    const int32_t* constraint_node;
    const int32_t* constraint_dir;
    const double* constraint_velocity;
    /* piecewise-linear time functions; table k holds function_npoints[k] points */
    int n_functions;
    const int32_t* function_npoints;
    const double* function_x;
    const double* function_y;
    /* concentrated nodal forces, flattened (node, dir, force, function); function
       -1 = Unit, k >= 0 = table k.  Applied in list order. */
    int n_nodal_forces;
    const int32_t* nodal_force_node;
    const int32_t* nodal_force_dir;
    const double* nodal_force_value;
    const int32_t* nodal_force_function;
    int n_materials;
    const MpmMaterial* materials;
} MpmDesc;

/* Particle fields (mpm_write_field / mpm_read_field). */
typedef enum MpmField {
    MPM_FIELD_LOC = 0,            /* float (n, ndim) */
    MPM_FIELD_VELOCITY = 1,       /* float (n, ndim) */
    MPM_FIELD_STRESS = 2,         /* float (n, 6) */
    MPM_FIELD_STRAIN = 3,         /* float (n, 6) */
    MPM_FIELD_DENSITY = 4,        /* float (n) */
    MPM_FIELD_VOLUME = 5,         /* float (n) */
    MPM_FIELD_MASS = 6,           /* float (n) */
    MPM_FIELD_VSC = 7,            /* float (n) volumetric_strain_centroid */
    MPM_FIELD_MATERIAL_ID = 8,    /* int32 (n) */
    MPM_FIELD_YOUNGS_MODULUS = 9, /* float (n) per-particle E (LinearElastic), write enables it */
    MPM_FIELD_ELEMENT_ID = 10,    /* int32 (n), read only */
    MPM_FIELD_MOMENTUM = 11,      /* float (n, ndim), read only: mass * velocity */
    MPM_FIELD_COUNT = 12
} MpmField;

/* Nodal fields (mpm_read_nodal_field / mpm_write_nodal_field). */
typedef enum MpmNodalField {
    MPM_NODE_MASS = 0,            /* float (Nn) */
    MPM_NODE_VELOCITY = 1,        /* float (Nn, ndim) */
    MPM_NODE_ACCELERATION = 2,    /* float (Nn, ndim) */
    MPM_NODE_MOMENTUM = 3         /* float (Nn, ndim), read only: mass * velocity */
} MpmNodalField;

/* Phases for mpm_run_phase (test and debugging entry). */
typedef enum MpmPhase {
    MPM_PHASE_NODAL_KINEMATICS = 0, /* scheme.py:22-29 (+ the step's volume reset) */
    MPM_PHASE_FORCES = 1,           /* USF: scheme.py:31-56 + element.py:305-329; USL: scheme.py:37-56 + element.py:305-329 */
    MPM_PHASE_PARTICLE_KINEMATICS = 2 /* particle.py:208-247 (USL: + scheme.py:31-35) */
} MpmPhase;

/* Library ABI version (MPM_ABI_VERSION). */
int mpm_abi_version(void);

/* Create a simulation on the current CUDA device.
 * Replaces Quadrilateral4Node.__init__ (diffmpm/element.py:626-690) and the
 * configuration part of MPMExplicit.__init__ (diffmpm/solver.py:24-80). */
int mpm_create(const MpmDesc* desc, MpmHandle** out);

/* Free every device buffer of the handle. */
int mpm_destroy(MpmHandle* h);

/* Message of the last failure on `h` (or of the last failed mpm_create when h is NULL). */
const char* mpm_last_error(const MpmHandle* h);

/* Set the particle population: `n` particles at `loc` (n, ndim) with material
 * ids (NULL = all 0).  Every other field takes the reference's initial value
 * (diffmpm/particle.py:53-71: zero velocity/stress/strain, density from the
 * material).  Replaces Particles.__init__ (diffmpm/particle.py:16-91). */
int mpm_set_particles(MpmHandle* h, int64_t n, const float* loc, const int32_t* material_id,
                      int on_device, void* stream);

/* Overwrite one particle field (original particle order). */
int mpm_write_field(MpmHandle* h, int field, const void* src, int on_device, void* stream);

/* Read one particle field in original particle order.  Replaces the output
 * assembly of MPMExplicit.solve_jit (diffmpm/solver.py:214-222). */
int mpm_read_field(MpmHandle* h, int field, void* dst, int on_device, void* stream);

/* Asynchronous output: enqueue on `stream` the copy of `nfields` particle
 * fields (original order, each as mpm_read_field lays it out, one after the
 * other) into the pinned host buffer `host_dst` of `host_dst_bytes` bytes,
 * and return at once with a ticket; mpm_output_wait(ticket) blocks until that
 * copy is in host memory and may be called from another host thread while
 * this one keeps stepping.  The copy needs 4 * np * (sum of the fields'
 * component counts) bytes; a smaller `host_dst_bytes` returns MPM_ERR_INVALID
 * before anything is enqueued.  At most 8 copies may be outstanding.
 * Replaces the host callback that writes the outputs of solve_jit every
 * out_steps steps (diffmpm/solver.py:187-210, writers.py:30-54). */
int mpm_output_enqueue(MpmHandle* h, int nfields, const int* fields, void* host_dst,
                       size_t host_dst_bytes, void* stream, int64_t* ticket);
int mpm_output_wait(MpmHandle* h, int64_t ticket);

/* Pinned host memory for mpm_output_enqueue. */
int mpm_host_alloc(size_t bytes, void** p);
int mpm_host_free(void* p);

/* Particle tractions (diffmpm/forces.py:26-41, mesh.py:60-77): `n` entries
 * (particle id, dir, traction, function: -1 Unit, k table k).  Replaces any
 * previous list. */
int mpm_set_tractions(MpmHandle* h, int n, const int64_t* pid, const int32_t* dir,
                      const double* traction, const int32_t* function, void* stream);

/* Particle velocity constraints: after the particle velocity update of every
 * step, the velocity of particle pid[i] (original order) in direction dir[i]
 * becomes velocity[i]; later entries win; n = 0 clears the list.  The
 * reference leaves this step as a TODO (diffmpm/scheme.py:67); this extension
 * mirrors the nodal Constraint (diffmpm/constraint.py:29-44) on particles. */
int mpm_set_particle_velocity_constraints(MpmHandle* h, int n, const int64_t* pid, const int32_t* dir,
                                          const double* velocity, void* stream);

/* Nodal state access (diffmpm/node.py:64-71). */
int mpm_read_nodal_field(MpmHandle* h, int field, float* dst, int on_device, void* stream);
int mpm_write_nodal_field(MpmHandle* h, int field, const float* src, int on_device, void* stream);

/* Sort particles by cell and run the volume set-up: element ids, element
 * volume, particle volume/size/mass (diffmpm/solver.py:81-85).  Must follow
 * mpm_set_particles before the first step. */
int mpm_initialize(MpmHandle* h, void* stream);

/* Advance `nsteps` explicit steps.  Replaces the body of solve_jit's
 * lax.fori_loop (diffmpm/solver.py:179-213) or of solve's loop
 * (diffmpm/solver.py:144-149), per desc.reinit_each_step. */
int mpm_step(MpmHandle* h, int nsteps, void* stream);

/* Step counter i (t = i * dt in the time functions, diffmpm/scheme.py:52-54). */
int mpm_get_step(const MpmHandle* h, int64_t* step);
int mpm_set_step(MpmHandle* h, int64_t step);

/* Run one phase of one step (for tests).  Steps that use this must run the
 * three phases in order. */
int mpm_run_phase(MpmHandle* h, int phase, void* stream);

/* Advance `nsteps` steps launching the three phase kernels directly (no graph)
 * with CUDA events between them, and return the summed device time of each
 * phase in ms_out[0..2] (nodal kinematics, forces, particle kinematics).  For
 * measurement; the state advances as with mpm_step. */
int mpm_time_phases(MpmHandle* h, int nsteps, float* ms_out, void* stream);

/* Steps per captured CUDA graph (default 100). */
int mpm_set_block_steps(MpmHandle* h, int steps);
/* Kernel builds of the step: the nodal-kinematics and USF G2P kernels for
 * nk_ctas / g2p_ctas resident CTAs per SM (2 or 3), and the forces kernel's
 * fast path (forces_lpc, see MpmTuning).  Results are the same bits either
 * way; only the speed differs (mpm_batch_autotune chooses them for a batch). */
int mpm_set_kernel_variant(MpmHandle* h, int nk_ctas, int g2p_ctas, int forces_lpc);

/* Tiles whose cells and ring of cells store no particle need only a node
 * update per step.  When a simulation has at least `min_empty` such tiles
 * (default 128), its step kernels are launched over the other tiles and one
 * kernel updates the empty tiles' nodes; otherwise every tile goes through
 * the step kernels.  Results are the same bits either way; 0 always splits,
 * INT_MAX never does.  No counterpart in the reference. */
int mpm_set_empty_split(MpmHandle* h, int min_empty);

/* Name of CUDA device `device` with its compute capability and SM count
 * (NUL-terminated, truncated to len bytes), the GPU part of the key under
 * which tuning results are cached.  No counterpart in the reference. */
int mpm_device_name(int device, char* name, int len);

/* Replace desc.gravity (the `gravity` argument of solve_jit / solve,
 * diffmpm/solver.py:116,159), so one handle serves solves with any gravity. */
int mpm_set_gravity(MpmHandle* h, double gx, double gy);

/* Number of particle re-sorts and rolled-back step blocks so far. */
int mpm_get_counters(const MpmHandle* h, int64_t* resorts, int64_t* rollbacks);

/* Differentiation.  The reference differentiates solve_jit with jax.grad
 * (examples/optim_1d.py:33-41,55 takes jax.value_and_grad of a loss of the
 * final velocities); these two calls are the hand-written reverse of the same
 * steps, for every configuration the forward runs: Quadrilateral4Node and
 * Linear1D meshes, LinearElastic, SimpleMaterial and Newtonian particles, USF
 * or USL, with or without the per-step volume set-up, particle tractions and
 * particle velocity constraints.
 *
 * mpm_record advances `nsteps` steps like mpm_step and keeps a checkpoint of
 * the full state every `checkpoint_steps` steps (and at the end); on a
 * Linear1D mesh it keeps every step's start state instead (checkpoint_steps
 * is not used). */
int mpm_record(MpmHandle* h, int nsteps, int checkpoint_steps, void* stream);

/* Gradient of a loss L(x_end, v_end) through the steps of the last
 * mpm_record, given dL/dx_end (n, ndim) and dL/dv_end (n, ndim; NULL = zero) in
 * original particle order.  Writes, in original particle order, any of
 * dL/dE (n; per-particle Young's modulus, or the material's modulus counted
 * per particle: the sum over a material's particles is dL/dE of that
 * material), dL/dx_0 (n, ndim) and dL/dv_0 (n, ndim) at the recorded start; NULL
 * outputs are skipped.  Each segment between checkpoints is re-run to rebuild
 * its per-step tape.  The handle is left at the recorded end state, so the
 * call may be repeated with other seeds; any call that changes the state
 * (step, write, set) in between makes it return MPM_ERR_STATE. */
int mpm_adjoint(MpmHandle* h, const float* dl_dloc, const float* dl_dvel, float* dl_dE,
                float* dl_dloc0, float* dl_dvel0, int on_device, void* stream);

/* Batches of independent simulations.  No counterpart in the reference, which
 * runs one simulation per solve; a batch advances many (of any mesh and
 * particle counts) with one kernel launch per phase per step for all of
 * them, captured in CUDA graphs of step blocks.  The handles must be
 * initialised, on one device, and share the scheme, volume set-up and
 * traction set-up; each keeps its own state, so mpm_read_field etc. work on
 * them as usual.  Destroy the batch before its handles (mpm_batch_destroy
 * does not touch them). */
typedef struct MpmBatch MpmBatch;

int mpm_batch_create(MpmHandle* const* sims, int n, MpmBatch** out);
int mpm_batch_destroy(MpmBatch* b);
/* Message of the last failure on b (NULL: of the last mpm_batch_create). */
const char* mpm_batch_last_error(const MpmBatch* b);
/* Number of simulations and of tiles (CTAs per phase launch). */
int mpm_batch_size(const MpmBatch* b, int* n, int* ntiles);
/* Whole-batch state transfers (a restart of every member from new initial
 * states without per-member round trips).  `src` / `dst` hold the members'
 * fields one after the other (member order; within a member the layout of
 * mpm_write_field / mpm_read_field / mpm_write_nodal_field); host memory is
 * copied in one transfer.  Writable particle fields: loc, velocity, stress,
 * strain, density, volumetric strain.  mpm_batch_restart sets every member's
 * step to 0 and re-runs its initialisation (re-sort, solve-semantics volume
 * set-up).  Replace per-simulation Particles / Nodes assignments and the
 * MPMExplicit constructor (diffmpm/particle.py:16-91, node.py:64-71,
 * solver.py:81-85) for all members at once. */
int mpm_batch_write_field(MpmBatch* b, int field, const void* src, int on_device, void* stream);
int mpm_batch_read_field(MpmBatch* b, int field, void* dst, int on_device, void* stream);
int mpm_batch_write_nodal_field(MpmBatch* b, int field, const float* src, int on_device, void* stream);
int mpm_batch_restart(MpmBatch* b, void* stream);

/* Advance every simulation by `nsteps` steps (as mpm_step does for one). */
int mpm_batch_step(MpmBatch* b, int nsteps, void* stream);
/* Steps per captured graph (default 100). */
int mpm_batch_set_block_steps(MpmBatch* b, int steps);
/* Tuning of a batch's step loop (no counterpart in the reference, which
 * runs one simulation per solve_jit):
 *   block_steps   steps per captured CUDA graph (a step block);
 *   resort_every  a simulation whose particles left their sort-cells is
 *                 re-sorted at the start of every resort_every-th block (in
 *                 between its drifted cells take the gathering path; a
 *                 particle two cells from its sort-cell rolls the block back
 *                 either way), so particles are re-sorted every
 *                 block_steps * resort_every steps at most;
 *   nk_ctas       CTAs per SM the nodal-kinematics kernel is built for (3:
 *                 40 registers a thread, or 2);
 *   g2p_ctas      the same for the USF G2P kernel;
 *   forces_lpc    the forces kernel's fast path: 0, a warp's lanes take
 *                 consecutive particles of a cell row and add their
 *                 contributions through shared memory; 1, each lane works
 *                 through the particles of its own cell in global memory;
 *                 2, the same on the cell row staged in shared memory by
 *                 16-byte copies, with the updated state copied back the
 *                 same way;
 *   ms_per_step   (output of mpm_batch_autotune) device time per step.
 * The builds and the re-sort cadence change no result beyond the last bits
 * of the re-sort schedule's summation order. */
typedef struct MpmTuning {
    int32_t block_steps;
    int32_t resort_every;
    int32_t nk_ctas;
    int32_t g2p_ctas;
    int32_t forces_lpc;
    float ms_per_step;
} MpmTuning;

/* Time `trial_steps` steps of the batch from its current state for
 * candidate tunings -- coordinate descent over the kernel builds
 * ({2, 3} x {2, 3} CTAs per SM, each of the three forces paths), the block length (10, 25, 50, 100, 200,
 * capped at trial_steps) and the re-sort cadence (1, 2, 4 blocks) --, apply
 * the fastest, put every simulation back in the state it had, and return the
 * choice in *best (may be NULL). */
int mpm_batch_autotune(MpmBatch* b, int trial_steps, MpmTuning* best, void* stream);
/* Apply a tuning (for example one read back from a cache of earlier
 * mpm_batch_autotune results), or read the current one. */
int mpm_batch_set_tuning(MpmBatch* b, const MpmTuning* tuning);
int mpm_batch_get_tuning(const MpmBatch* b, MpmTuning* tuning);

/* mpm_record / mpm_adjoint for every simulation of a batch at once: one
 * launch per re-run step and per reverse pass for all of them.  The arrays
 * hold one pointer per simulation (batch order); dl_dvel and the outputs may be
 * NULL as a whole or per entry. */
int mpm_batch_record(MpmBatch* b, int nsteps, int checkpoint_steps, void* stream);
int mpm_batch_adjoint(MpmBatch* b, const float* const* dl_dloc, const float* const* dl_dvel,
                      float* const* dl_dE, float* const* dl_dloc0, float* const* dl_dvel0,
                      int on_device, void* stream);

/* Largest mesh (nx * ny elements) mpm_volume_setup_noalloc accepts. */
#define MPM_NOALLOC_MAX_ELEMENTS (1 << 20)

/* Particle volume set-up that allocates no device memory.  No counterpart in
 * the reference: it is the no-allocation form of this library's set-up
 * (element id, V = V_el / particles in the element, mass = V * density, the
 * values mpm_initialize and mpm_read_field(ELEMENT_ID / VOLUME / MASS) give),
 * for callers that cannot call cudaMalloc -- a JAX/XLA FFI handler, whose
 * buffers come from XLA's allocator, or an application whose framework owns the
 * device memory pool.  All pointers are device memory: loc (n, 2), density (n)
 * in; element_id (n), volume (n), mass (n) out.  One difference from the
 * allocating set-up: a particle outside the mesh (including one exactly on
 * its top or right edge) gets element id -1 and zero volume and mass, where
 * mpm_initialize refuses the whole population with MPM_ERR_OUT_OF_MESH.
 * The per-element counters live in a fixed 4 MiB device array, so the mesh may
 * have at most MPM_NOALLOC_MAX_ELEMENTS elements (larger meshes return
 * MPM_ERR_INVALID).  That array stays resident on every GPU that loads the
 * library.  The first call on a device (with that device current) looks up
 * the array's address and keeps it for the life of the process; make that
 * first call before any stream capture, and do not call this entry point
 * again on a device after cudaDeviceReset (the kept address would be stale).
 * All calls share the array, so calls that overlap on the GPU race; order
 * them.  Errors are reported through mpm_last_error(NULL). */
int mpm_volume_setup_noalloc(int nx, int ny, double hx, double hy, int64_t n, const float* loc,
                             const float* density, int32_t* element_id, float* volume,
                             float* mass, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* DIFFMPM_GB300_H */
