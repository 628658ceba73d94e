// Batch of simulation handles (mpm_batch.cu) and the host helpers the
// batched adjoint (mpm_adjoint.cu) shares with the batched step.
#pragma once
#include <map>
#include <string>
#include <vector>

#include "mpm_handle.h"

namespace mpm {
struct BatchAdjoint;   // scratch of the batched adjoint (mpm_adjoint.cu)
}

struct MpmBatch {
    int device = 0;
    std::vector<MpmHandle*> sims;
    mpm::StepConfig cfg{};
    const mpm::SimDev** d_sims = nullptr;
    mpm::TileDesc* d_tdescs = nullptr;  // records of the active tiles, refreshed per block
    mpm::TileDesc* d_edescs = nullptr;  // records of the empty tiles (node updates only)
    int4* d_act_list = nullptr;         // the tile list split by launch_classify_tiles_batch
    int4* d_emp_list = nullptr;
    int* d_tflags = nullptr;
    int* d_tcounts = nullptr;           // [active, empty]
    int* h_tcounts = nullptr;           // pinned
    int nact = 0, nemp = 0;
    void* d_stage = nullptr;            // staging of whole-batch field transfers
    size_t stage_bytes = 0;
    mpm::Control** d_ctls = nullptr;
    int4* d_tiles = nullptr;
    int ntiles = 0;
    mpm::Control* d_status = nullptr;
    mpm::Control* h_status = nullptr;   // pinned
    int block_steps = 100;
    int resort_every = 1;               // re-sort a drifted simulation every this many blocks
    std::vector<int> since_resort;      // blocks each simulation has run since it drifted
    cudaStream_t cap = nullptr;
    std::map<int64_t, cudaGraphExec_t> graphs;   // keyed by steps and tile counts
    mpm::SegBuf segbuf;
    std::vector<mpm::Checkpoint> tune;  // per-simulation state saved by the autotuner
    mpm::BatchAdjoint* badj = nullptr;
    std::string err;
};

namespace mpm {
namespace batch {

int bfail(MpmBatch* b, int code, const char* fmt, ...);
// A failure reported on simulation i's handle, copied to the batch.
int from_sim(MpmBatch* b, int i, int code);
int check_ready(MpmBatch* b);
// Split the batch's tiles into active and empty ones and write their records
// (descriptor, row starts, occupancy) for the current descriptors and sorts;
// needed whenever a descriptor or a sort changed.  Waits for the counts, so
// not inside a stream capture.
int prepare_tiles(MpmBatch* b, cudaStream_t s);
// n steps of every simulation as 3n batched launches over the active tiles
// plus one over the empty tiles per step (no status handling).
int launch_batch_steps(MpmBatch* b, int n, cudaStream_t s);
// Gather every control block into b->h_status and clear the status words.
int read_statuses(MpmBatch* b, cudaStream_t s);
// Advance every simulation by nsteps steps in blocks (re-sorts, snapshots,
// graphs, rollbacks).
int batch_steps(MpmBatch* b, int nsteps, cudaStream_t s);

#define BCK(b, call)                                                                          \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return ::mpm::batch::bfail(b, MPM_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

#define BTRY(b, i, x)                                                \
    do {                                                             \
        int r_ = (x);                                                \
        if (r_ != MPM_OK) return ::mpm::batch::from_sim(b, i, r_);   \
    } while (0)

}  // namespace batch

void batch_adjoint_free(MpmBatch* b);

}  // namespace mpm
