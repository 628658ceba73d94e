// Reverse (adjoint) passes of the explicit MPM step, USF or USL, with the
// per-step volume set-up of solve_jit (diffmpm/solver.py:81-85, 100-111,
// 179-213).
//
// The reverse of one USF step runs four launches over the step's tape (the
// particle state at the step start and the nodal values the forward step
// produced), in the reverse order of the forward phases:
//   1. node pass      transposed G2P (v-hat, a-hat adjoints gathered to the
//                     nodes) and the reverse nodal update (a = f/m, v += a dt,
//                     constraints, flush); also the per-cell particle counts
//   2. particle pass  reverse of the forces (internal + external) and of the
//                     USF strain, volume, density and stress update
//   3. node pass      transposed strain-rate gather (nodal-velocity adjoint)
//                     and the reverse nodal velocity p/m with constraints
//   4. particle pass  reverse of the mass and momentum P2G
// A USL step (stress update after G2P, from the updated nodal velocities)
// runs two more first: U, a particle pass reversing that stress update, and
// G, the node pass gathering its strain-rate adjoints into the nodal
// velocity adjoint that pass 1 adds; then passes 1-4 with the forces of pass
// 2 on the start-of-step stress and no gather in pass 3.
// Every node sum is formed in a fixed order (the four cells around the node,
// particles of a cell in storage order), so the adjoint is deterministic.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "mpm_types.h"

namespace mpm {

// Everything one reverse step reads and writes; passed by value.
struct AdjStep {
    // mesh and run constants
    int nx, ny, np;
    float hx, hy, dt, vol_el, gx, gy;
    int velocity_update;
    const uint16_t* ncons;
    const MatDev* mats;
    // sort epoch of the step: cell starts, material ids and per-particle E
    const int* cstart;
    const uint8_t* mat;
    const float* E;
    // tape: particle state at the step start (storage order), drift flags,
    // nodal mass, velocity after phase 1 (vA), velocity and acceleration after
    // the nodal update (vB, aB)
    const float *x, *y, *vx, *vy, *sxx, *syy, *szz, *sxy, *rho;
    const uint8_t* cflag;
    const float *nm, *nvax, *nvay, *nvbx, *nvby, *nax, *nay;
    // adjoint of the particle state (in: end of step; out: start of step) and
    // the accumulated dL/dE per particle
    float *lx, *ly, *lvx, *lvy, *lsxx, *lsyy, *lszz, *lsxy, *lrho, *lE;
    // per-particle adjoints of the strain rates and centroid rates (USF:
    // pass 2 -> 3; USL: pass U -> G and 2)
    float *r0b, *r1b, *r3b, *c0b, *c1b;
    // nodal adjoints: force, mass and phase-1 velocity from the nodal update
    // (pass 1 -> 2, 3; USL pass G leaves its vB-bar in vabx, vaby for pass 1),
    // momentum and total mass (pass 3 -> 4)
    float *fbx, *fby, *mb, *vabx, *vaby;
    float *qbx, *qby, *mbt;
    int* cnt;              // particles per cell at the step start (pass 1 -> 2, 4)
    // particle tractions (tr_fn null when the run has none): function code and
    // traction per particle and direction in the epoch's storage order, the
    // function tables, and the step number of the step being reversed
    const int8_t* tr_fn;
    const float* tr_tau;
    // particle velocity constraint codes (2 per particle, epoch storage
    // order; null when the run has none): a constrained velocity component
    // is set after G2P and passes no adjoint
    const uint8_t* pvc;
    // solve semantics (reinit 0: no per-step volume set-up): the volume at the
    // step start (tape), the constant mass and size (epoch order) and the
    // volume adjoint (in: end of step; out: start of step)
    int reinit;
    const float *vol, *mass, *psize;
    float* lvol;
    // centroid volumetric strain at the step start (tape; null unless a
    // material reads it: Newtonian) and its adjoint
    const float* vsc;
    float* lvsc;
    const int* fn_off;
    const float *fn_x, *fn_y;
    int step;
    // tape slot strides (particles, nodes, cells) for batched launches
    long long sp, sn, sc;
};

// The passes of one reverse step: node passes over the forward kernels' tile
// list, particle passes over the particles.
cudaError_t launch_rev_step(const AdjStep& A, bool usl, bool trac, const int4* tiles, int ntiles,
                            cudaStream_t s);

// Batches: table[i] = bases[i] with the tape pointers at slot t; then the
// passes over every simulation: passes 1 and 3 over the batch's tile list
// (tile t of simulation tiles[t].x), passes 2 and 4 with CTA b on simulation
// part_blocks[b].x, particles part_blocks[b].y * 256 .. + 255.
constexpr int ADJ_BLOCK = 256;
// Particles of one simulation per block of the batched particle passes: the
// block copies the simulation's arguments once and walks ADJ_ITER chunks.
constexpr int ADJ_ITER = 4;
cudaError_t launch_adj_table(const AdjStep* bases, int n, int t, AdjStep* table, cudaStream_t s);
// `pvc`: some simulation of the batch has particle velocity constraints.
// `newt`: some simulation of the batch has Newtonian particles.
cudaError_t launch_rev_batch(const AdjStep* table, bool usl, bool trac, bool pvc, bool reinit, bool newt,
                             const int4* tiles, int ntiles, const int2* part_blocks, int n_part_blocks,
                             cudaStream_t s);

}  // namespace mpm
