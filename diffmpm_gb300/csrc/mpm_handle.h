// Host-side state of one simulation handle and the host helpers shared by
// the forward step (mpm_abi.cu) and the adjoint (mpm_adjoint.cu).
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/diffmpm_gb300.h"
#include "mpm_kernels.h"
#include "mpm_types.h"

namespace mpm {

// One buffer set of the cell-sorted particle arrays (a re-sort gathers into
// the other set and swaps).
struct PSet {
    float *x = nullptr, *y = nullptr, *vx = nullptr, *vy = nullptr;
    float *sxx[2] = {}, *syy[2] = {}, *szz[2] = {}, *sxy[2] = {};
    float *exx = nullptr, *eyy = nullptr, *exy = nullptr;
    float *rho[2] = {}, *vsc[2] = {}, *vol[2] = {};
    float *mass = nullptr, *psize = nullptr, *E = nullptr, *tr_tau = nullptr;
    uint8_t* mat = nullptr;
    int8_t* tr_fn = nullptr;
    uint8_t* pvc = nullptr;     // particle velocity constraint codes (2 per particle)
    int* pid = nullptr;
};

struct AdjointState;   // checkpoints, tape and adjoint arrays (mpm_adjoint.cu)
struct LineAdjoint;    // the 1-D step's full tape and adjoint arrays (mpm_line_adjoint.cu)

// Full copy of the state of one simulation that steps and re-sorts change:
// the particle arrays (storage order, current ping-pong parity), material ids,
// traction and velocity-constraint codes, cell starts, drift flags, the
// persistent nodal velocity and the control block.
struct Checkpoint {
    int64_t step = 0;
    bool needs_resort = false;
    std::vector<float*> f;   // movable_f32(.., false) of the particle set
    uint8_t* mat = nullptr;
    int8_t* tr_fn = nullptr;    // particle tractions (2 per particle), when present
    float* tr_tau = nullptr;
    uint8_t* pvc = nullptr;     // particle velocity constraint codes (2 per particle), when present
    int* cstart = nullptr;
    uint8_t* cflag = nullptr;
    float *nvbx = nullptr, *nvby = nullptr;
    Control* ctl = nullptr;
};

// Device tables of a segmented copy (grown on demand) and the size of the
// list last uploaded.
struct SegBuf {
    CopySeg* segs = nullptr;
    unsigned* first = nullptr;
    CopyChunk* blk = nullptr; // chunk table of the copy kernels
    size_t cap = 0;
    size_t blk_cap = 0;
    int nseg = 0;
    unsigned nblocks = 0;
};

}  // namespace mpm

struct MpmHandle {
    int device = 0;
    // configuration
    int ndim = 2, nx = 0, ny = 0;
    float hx = 0, hy = 0, dt = 0, gx = 0, gy = 0, vol_el = 0;
    bool usl = false, reinit = true;
    int velocity_update = 0;
    int nmat = 0;
    std::vector<mpm::MatDev> mats;
    // device tables
    mpm::MatDev* d_mats = nullptr;
    float* d_cons_vel = nullptr;
    uint16_t* d_ncons = nullptr;
    int* d_cnf_ptr = nullptr;
    int8_t* d_cnf_dir = nullptr;
    float* d_cnf_val = nullptr;
    int8_t* d_cnf_fn = nullptr;
    int nfn = 0;
    int* d_fn_off = nullptr;
    float *d_fn_x = nullptr, *d_fn_y = nullptr;
    // nodes
    int nn = 0;
    float *nm = nullptr, *nvax = nullptr, *nvay = nullptr, *nvbx = nullptr, *nvby = nullptr;
    float *nax = nullptr, *nay = nullptr;
    // cells
    int ncell = 0;
    int* cstart[2] = {};
    int cs_cur = 0;
    uint8_t* cflag = nullptr;
    mpm::SortScratch sw{};
    // particles
    int64_t np = -1;
    mpm::PSet ps[2];
    int pcur = 0;
    float* passive = nullptr;   // original order, 5 per particle: s_yz s_xz e_zz e_yz e_xz
    bool has_trac = false, has_E = false;
    // snapshot of the mutable state at a block start
    std::vector<float*> snap_f;
    uint8_t* snap_cflag = nullptr;
    float *snap_nvbx = nullptr, *snap_nvby = nullptr;
    mpm::Control* snap_ctl = nullptr;
    mpm::SegBuf segbuf;
    // descriptors
    mpm::SimDev hs{};
    mpm::SimDev* ds = nullptr;
    mpm::Control* ctl = nullptr;
    mpm::Control* h_ctl = nullptr;   // pinned mirror
    int4* dtiles = nullptr;
    int ntiles = 0;
    // the tiles split by launch_classify_tiles (active: the step kernels'
    // grid; empty: node updates only), refreshed at the start of every
    // launched sequence
    int4* d_active = nullptr;
    int4* d_empty = nullptr;
    int* d_tile_flags = nullptr;
    int* d_tile_counts = nullptr;    // [active, empty]
    int* h_tile_counts = nullptr;    // pinned mirror
    int nact = 0, nemp = 0;          // the step kernels' and the empty-node kernel's grids
    const int4* step_tiles = nullptr; // the step kernels' list: d_active after a split, else dtiles
    int64_t step = 0;
    // staging and pointer tables
    void* stage = nullptr;
    size_t stage_bytes = 0;
    float** d_ptrs = nullptr;
    int* line_eid = nullptr;         // 1-D: element of each storage slot this step
    // asynchronous output (mpm_output_enqueue): its own staging buffer and a
    // ring of events, one per outstanding copy
    static constexpr int OUT_SLOTS = 8;
    void* out_stage = nullptr;
    size_t out_stage_bytes = 0;
    cudaEvent_t out_ev[OUT_SLOTS] = {};
    int64_t out_tickets = 0;
    // graphs
    cudaStream_t cap = nullptr;
    std::map<int64_t, cudaGraphExec_t> graphs;   // keyed by steps and the tile counts
    bool graphs_trac = false;
    uint64_t graph_gen = 0;            // bumped whenever the step graphs are dropped
    bool has_pvc = false;              // particle velocity constraints set
    float* d_pvc_vel = nullptr;
    bool initialized = false, needs_resort = false;
    int block_steps = 100;
    int nk_ctas = 3, g2p_ctas = 2;     // kernel builds (StepConfig), set by mpm_set_kernel_variant
    int forces_lpc = 0;
    int empty_split_min = mpm::EMPTY_SPLIT_MIN;   // mpm_set_empty_split
    int64_t resorts = 0, rollbacks = 0;
    // differentiation (null until mpm_record); gen counts state changes
    mpm::AdjointState* adj = nullptr;
    mpm::LineAdjoint* line_adj = nullptr;   // 1-D recording (mpm_line_adjoint.cu)
    uint64_t gen = 0;
    std::vector<void*> allocs;
    std::string err;
};

namespace mpm {
namespace host {

int fail(MpmHandle* h, int code, const char* fmt, ...);

#define CK(h, call)                                                                          \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return ::mpm::host::fail(h, e_ == cudaErrorMemoryAllocation ? MPM_ERR_NOMEM      \
                                                                        : MPM_ERR_CUDA,      \
                                     "%s: %s (%s:%d)", #call, cudaGetErrorString(e_),        \
                                     __FILE__, __LINE__);                                    \
    } while (0)

#define TRY(x)                       \
    do {                             \
        int r_ = (x);                \
        if (r_ != MPM_OK) return r_; \
    } while (0)

template <class T>
int dalloc(MpmHandle* h, T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    void* v = nullptr;
    cudaError_t e = cudaMalloc(&v, count * sizeof(T));
    if (e != cudaSuccess)
        return fail(h, MPM_ERR_NOMEM, "cudaMalloc(%zu bytes): %s", count * sizeof(T),
                    cudaGetErrorString(e));
    h->allocs.push_back(v);
    *p = static_cast<T*>(v);
    return MPM_OK;
}

void dfree(MpmHandle* h, void* p);
inline cudaStream_t S(void* s) { return static_cast<cudaStream_t>(s); }

void drop_graphs(MpmHandle* h);
int upload_desc(MpmHandle* h);
void bind_particles(MpmHandle* h);
int parity(const MpmHandle* h);
std::vector<float**> movable_f32(MpmHandle* h, PSet& p, bool for_snapshot);
int ensure_stage(MpmHandle* h, size_t bytes);
int sync(MpmHandle* h, cudaStream_t s);
int read_ctl(MpmHandle* h, cudaStream_t s);
int clear_status(MpmHandle* h, cudaStream_t s);
int resort(MpmHandle* h, cudaStream_t s);
// n steps from ctl->step (the tiles classified for the current sort).
int launch_steps(MpmHandle* h, int n, cudaStream_t s);
// Phase `phase` (0 nodal kinematics, 1 forces, 2 G2P) of step ctl->step + k.
int launch_phase(MpmHandle* h, int phase, int k, cudaStream_t s);
// The step kernels' tile list and grids (step_tiles, nact, nemp) for the
// current sort; call before a sequence of launch_phase (it waits for the
// counts, so not inside a stream capture).
int classify_tiles(MpmHandle* h, cudaStream_t s);
// Graph-cache key of a step sequence: its length and the grids it launches.
int64_t seq_key(const MpmHandle* h, int n);
int check_status(MpmHandle* h, int& st);
int take_snapshot(MpmHandle* h, cudaStream_t s);
int replay_block(MpmHandle* h, int64_t step0, int B, int& st, cudaStream_t s);
// Where a recorded 1-D step copies its start state (x, v, sxx, syy, szz, sxy,
// rho, volume, centroid volumetric strain in storage order, the storage ->
// original map and the element starts) and its nodal results (mass, velocity
// after kinematics, velocity and acceleration after the update).
struct LineTapeSlot {
    float* p[9];
    int* pid;
    int* cs;
    float* n[4];
};
int line_step(MpmHandle* h, cudaStream_t s, const LineTapeSlot* tape = nullptr);   // mpm_line.cu
int line_setup_volume(MpmHandle* h, cudaStream_t s);
int to_device(MpmHandle* h, const void* src, size_t bytes, int on_device, cudaStream_t s,
              const void** dsrc);
int ncomp_of(const MpmHandle* h, int field);
// Particle field I/O on stream s without waiting (mpm_abi.cu): a float field
// from device memory (original order), and any readable field to device memory.
int write_float_field(MpmHandle* h, int field, const float* d, cudaStream_t s);
int keep_parity_data(MpmHandle* h, int64_t step);
int gather_field(MpmHandle* h, int field, void* d, cudaStream_t s);


// Whole-state copies as segment lists (mpm_state.cu).  The snapshot of a step
// block goes to the handle's snap_* arrays; a checkpoint to its own arrays.
// A restore first sets the step counter (which selects the ping-pong parity
// the data goes to) and needs_resort from the saved values.
void snapshot_segments(MpmHandle* h, bool save, std::vector<CopySeg>& out);
int checkpoint_alloc(MpmHandle* h, Checkpoint& c);
void checkpoint_free(MpmHandle* h, Checkpoint& c);
void checkpoint_segments(MpmHandle* h, Checkpoint& c, bool save, std::vector<CopySeg>& out);
// Copy the segments in one launch on stream s (tables kept in `buf`, which
// owns its device memory; errors are reported on h).
int run_segments(MpmHandle* h, SegBuf& buf, const std::vector<CopySeg>& segs, cudaStream_t s);
// Upload only (launch later, possibly many times, with launch_copy_segments).
int upload_segments(MpmHandle* h, SegBuf& buf, const std::vector<CopySeg>& segs, cudaStream_t s);
void segbuf_free(SegBuf& buf);

}  // namespace host

// Adjoint bookkeeping (mpm_adjoint.cu): release the adjoint state of a handle;
// note a re-sort at the current step while mpm_record runs.
void adjoint_free(MpmHandle* h);
void line_adjoint_free(MpmHandle* h);
int line_record(MpmHandle* h, int nsteps, cudaStream_t s);
int line_adjoint(MpmHandle* h, const float* dl_dloc, const float* dl_dvel, float* dl_dE,
                 float* dl_dloc0, float* dl_dvel0, int on_device, cudaStream_t s);
void adjoint_note_resort(MpmHandle* h);

}  // namespace mpm
