// Host-side launchers of the MPM kernels (implemented in mpm_kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <cmath>
#include <string>
#include "mpm_types.h"

namespace mpm {

// Element volume of an hx x hy Quadrilateral4Node element by the reference's
// formula in float32 (diffmpm/element.py:903-909), on the host.
inline float element_volume(float hx, float hy) {
    const float a = hy, c = hy, b = hx, d = hx;
    const float p = std::sqrt(a * a + b * b), q = p;
    const float t = ((a * a + c * c) - b * b) - d * d;
    const float x = (((4.0f * p) * p) * q) * q - t * t;
    return 0.25f * std::sqrt(x);
}

struct StepConfig {
    bool usl;          // scheme: USL (else USF)
    bool reinit;       // solve_jit semantics: volume/mass reset each step
    bool traction;     // particle tractions present
    // resident CTAs per SM the nodal kinematics and USF G2P kernels are
    // built for: 3 (40 registers a thread) or 2 (up to 64)
    int nk_ctas = 3;
    int g2p_ctas = 2;
    // forces kernel fast path: particle per lane with row slots (0), lane
    // per cell (1), particle per lane on a staged row (2); the same bits
    // every way
    int forces_lpc = 0;
};

// One explicit step = three launches over the (active) tile list.  The descriptor is
// passed by value (a __grid_constant__ kernel parameter), so a captured graph
// holds the descriptor current at capture time.
cudaError_t launch_nodal_kinematics(const StepConfig& c, const SimDev& S, const int4* tiles,
                                    int ntiles, Control* ctl, int k, cudaStream_t s);
cudaError_t launch_forces(const StepConfig& c, const SimDev& S, const int4* tiles, int ntiles,
                          Control* ctl, int k, cudaStream_t s);
cudaError_t launch_particle_kinematics(const StepConfig& c, const SimDev& S, const int4* tiles,
                                       int ntiles, Control* ctl, int k, cudaStream_t s);
// Split the tile list into active tiles (cells or their ring store a
// particle; the step kernels' grid) and empty ones (node updates only,
// k_empty_nodes), in tile order, both padded to ntiles entries with
// (-1, 0, 0, 0), and write their counts to counts[0..1]; flags is ntiles
// ints of scratch.  Valid until the sort changes.
cudaError_t launch_classify_tiles(const SimDev& S, const int4* tiles, int ntiles, int* flags, int4* active,
                                  int4* empty, int* counts, cudaStream_t s);
// A single simulation launches its empty tiles apart only when it has at
// least this many (mpm_set_empty_split changes it per handle).
constexpr int EMPTY_SPLIT_MIN = 128;
// Grid of a launch over `count` tiles of such a list: the count rounded up to
// a multiple of TILE_GRID_QUANTUM (at most the list's length), so that the
// captured graphs, keyed by their grids, serve the small changes of the
// counts that re-sorts bring; the CTAs past the count read a (-1, ...) entry
// and return.
constexpr int TILE_GRID_QUANTUM = 64;
inline int tile_grid(int count, int ntiles) {
    if (count <= 0) return 0;
    const int q = (count + TILE_GRID_QUANTUM - 1) / TILE_GRID_QUANTUM * TILE_GRID_QUANTUM;
    return q < ntiles ? q : ntiles;
}
// The step's node updates of the empty tiles (before the nodal kinematics).
cudaError_t launch_empty_nodes(const SimDev& S, const int4* empty, int ntiles, Control* ctl, int k,
                               cudaStream_t s);
// The same for a batch: tiles of every simulation (sims[tile.x]); the empty
// tiles' records (launch_gather_tiles of the empty list).
cudaError_t launch_classify_tiles_batch(const SimDev* const* sims, const int4* tiles, int ntiles, int* flags,
                                        int4* active, int4* empty, int* counts, cudaStream_t s);
cudaError_t launch_empty_nodes_batch(const TileDesc* td, int ntiles, int k, cudaStream_t s);
// The kernels above work on step (ctl->step + k); these advance the counter
// once a sequence of steps has been launched.
cudaError_t launch_advance_step(Control* ctl, int by, cudaStream_t s);
cudaError_t launch_advance_steps(Control* const* ctls, int n, int by, cudaStream_t s);

// The same three phases for a batch of simulations in one launch each: tile
// t works on simulation tiles[t].x, whose descriptor is sims[tiles[t].x] and
// whose step counter and status are in ctls[tiles[t].x].
// out[t] = {tiles[t], ctls[tiles[t].x], *sims[tiles[t].x], row starts,
// occupancy} for t < ntiles (only out[t].T for a tile (-1, ...)).
cudaError_t launch_gather_tiles(const SimDev* const* sims, Control* const* ctls, const int4* tiles,
                                int ntiles, TileDesc* out, cudaStream_t s);
cudaError_t launch_nodal_kinematics_batch(const StepConfig& c, const TileDesc* td, int ntiles,
                                          int k, cudaStream_t s);
cudaError_t launch_forces_batch(const StepConfig& c, const TileDesc* td, int ntiles, int k,
                                cudaStream_t s);
cudaError_t launch_particle_kinematics_batch(const StepConfig& c, const TileDesc* td, int ntiles,
                                             int k, cudaStream_t s);

// Re-sort of one simulation's particles by current cell, stable in storage order.
struct SortScratch {
    int* count;        // ncell + 1 (last bucket: particles outside the mesh)
    int* cursor;       // ncell + 1
    int* key;          // np
    int* perm;         // np
    int* block_sums;   // ceil((ncell + 2) / 1024) + 1
};
cudaError_t launch_resort_keys(const SimDev* sim, int np, int nx, int ny, float hx, float hy,
                               const SortScratch& w, Control* ctl, cudaStream_t s);
cudaError_t launch_exclusive_scan(const int* in, int* out, int n, int* block_sums, cudaStream_t s);
cudaError_t launch_resort_place(int np, const int* start, const SortScratch& w, cudaStream_t s);
cudaError_t launch_resort_segsort(int nbucket, const int* start, const SortScratch& w,
                                  cudaStream_t s);

// dst[i] = src[perm[i]] for 4-byte and 1-byte elements.
cudaError_t launch_gather_u32(const uint32_t* src, uint32_t* dst, const int* perm, int n,
                              cudaStream_t s);
cudaError_t launch_gather_u8(const uint8_t* src, uint8_t* dst, const int* perm, int n,
                             cudaStream_t s);
cudaError_t launch_gather_pair_u32(const uint32_t* src, uint32_t* dst, const int* perm, int n,
                                   cudaStream_t s);
cudaError_t launch_gather_pair_u8(const uint8_t* src, uint8_t* dst, const int* perm, int n,
                                  cudaStream_t s);

// Solve-semantics volume set-up after a sort (V = V_el / count, m = V rho, size = sqrt V).
cudaError_t launch_setup_volume(const SimDev* sim, int np, int parity, cudaStream_t s);

// Field transfer between original order (AoS, ncomp per particle) and storage order (SoA).
// comp_ptrs: device array of ncomp float* (storage order); pid: storage -> original.
cudaError_t launch_scatter_out(const float* const* comp_ptrs, int ncomp, const int* pid, int np,
                               float* out, cudaStream_t s);
cudaError_t launch_gather_in(float* const* comp_ptrs, int ncomp, const int* pid, int np,
                             const float* in, cudaStream_t s);
cudaError_t launch_gather_in_u8(uint8_t* dst, const int* pid, int np, const int32_t* in,
                                cudaStream_t s);
cudaError_t launch_scatter_out_u8(const uint8_t* src, const int* pid, int np, int32_t* out,
                                  cudaStream_t s);

// Derived per-particle outputs in original order: element id, volume, mass
// (solve_jit semantics: the volume set-up at the current positions), momentum.
// 1-D (mpm_line.cu): buckets ordered by original index; element per storage slot
cudaError_t launch_line_segsort(int nbucket, const int* start, int* perm, const int* pid, cudaStream_t s);
cudaError_t launch_line_eid(const int* cstart, int nx, int* eid, cudaStream_t s);
cudaError_t launch_derived_out(const SimDev* sim, int ndim, int np, int parity, bool reinit, int what,
                               const int* pid, void* out, cudaStream_t s);

// Interleave / de-interleave nodal vectors.
cudaError_t launch_interleave2(const float* a, const float* b, int n, float* out, cudaStream_t s);
cudaError_t launch_deinterleave2(const float* in, int n, float* a, float* b, cudaStream_t s);
cudaError_t launch_node_momentum(const float* m, const float* vx, const float* vy, int n,
                                 float* out, cudaStream_t s);

// Copy of many device-memory segments in one launch (snapshots and checkpoints
// of whole batches, the adjoint's tape).  Segment i is cut into chunks of
// COPY_CHUNK bytes, chunks first[i] .. first[i+1]-1, first[nseg] being their
// number.  The chunk table (source, destination and length of every chunk)
// is formed on the device once per upload (launch_chunk_table), so a CTA of
// the copy kernel starts its chunk after one dependent load.  The
// destination of a launch with slot t is dst + t * dst_step.
struct CopySeg {
    const void* src;
    void* dst;
    unsigned long long bytes;
    unsigned long long dst_step;
};
struct CopyChunk {
    const char* src;
    char* dst;
    unsigned long long dst_step;
    unsigned long long bytes;
};
constexpr unsigned COPY_CHUNK = 16384;
cudaError_t launch_chunk_table(const CopySeg* segs, const unsigned* first, int nseg, unsigned nchunks,
                               CopyChunk* chunks, cudaStream_t s);
cudaError_t launch_copy_segments(const CopyChunk* chunks, unsigned nchunks, int t, cudaStream_t s);
// *mismatch += number of differing 16-byte words or tail bytes between src and dst.
cudaError_t launch_compare_segments(const CopyChunk* chunks, unsigned nchunks, int* mismatch,
                                    cudaStream_t s);

// out[i] = *ctls[i], then ctls[i]->status = 0, for i < n.
cudaError_t launch_gather_status(Control* const* ctls, int n, Control* out, cudaStream_t s);

// Set the calling thread's message returned by mpm_last_error(NULL).
void set_thread_error(const std::string& msg);

}  // namespace mpm
