// Batches: many independent simulations advanced together, one launch per
// phase per step for all of them (and one for all their empty tiles).
//
// A batch groups simulation handles of one configuration (scheme, volume
// set-up, tractions) on one GPU.  Their tiles form one tile list, each tile
// tagged with its simulation's index.  Before every step block one kernel
// classifies the tiles (active / empty) and writes a record per tile: the
// tile, its simulation's control pointer, a copy of the simulation's
// descriptor (the handle's device copy, which a re-sort updates in place) and
// the tile's row starts; the batched kernels read their tile's record, so a
// captured graph of a step block stays valid across re-sorts.  Per block:
// re-sort the simulations that drifted, snapshot all of them (one segmented
// copy), refresh the records, run the block graph, gather every status word
// in one copy; a simulation whose particle drifted two cells is rolled back
// and replayed alone, step by step.
// No counterpart in the reference, which runs one simulation per solve.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <map>
#include <set>
#include <string>
#include <vector>

#include "mpm_batch.h"

using namespace mpm;
using namespace mpm::host;

namespace {
thread_local std::string g_batch_create_error;
}  // namespace

namespace mpm {
namespace batch {

int bfail(MpmBatch* b, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (b) b->err = buf;
    else g_batch_create_error = buf;
    return code;
}

// A failure reported on simulation i's handle, copied to the batch.
int from_sim(MpmBatch* b, int i, int code) {
    return bfail(b, code, "simulation %d: %s", i, b->sims[i]->err.c_str());
}

void drop_batch_graphs(MpmBatch* b) {
    for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
    b->graphs.clear();
}

int prepare_tiles(MpmBatch* b, cudaStream_t s) {
    // the descriptors and row starts change only between step blocks
    // (re-sorts, set-up calls): one record per tile and block lets a CTA fetch
    // its tile, descriptor, control pointer and row starts in one read
    BCK(b, launch_classify_tiles_batch(b->d_sims, b->d_tiles, b->ntiles, b->d_tflags, b->d_act_list,
                                       b->d_emp_list, b->d_tcounts, s));
    BCK(b, launch_gather_tiles(b->d_sims, b->d_ctls, b->d_act_list, b->ntiles, b->d_tdescs, s));
    BCK(b, launch_gather_tiles(b->d_sims, b->d_ctls, b->d_emp_list, b->ntiles, b->d_edescs, s));
    BCK(b, cudaMemcpyAsync(b->h_tcounts, b->d_tcounts, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    BCK(b, cudaStreamSynchronize(s));
    b->nact = tile_grid(b->h_tcounts[0], b->ntiles);
    b->nemp = tile_grid(b->h_tcounts[1], b->ntiles);
    return MPM_OK;
}

int launch_batch_steps(MpmBatch* b, int n, cudaStream_t s) {
    for (int i = 0; i < n; ++i) {
        BCK(b, launch_empty_nodes_batch(b->d_edescs, b->nemp, i, s));
        BCK(b, launch_nodal_kinematics_batch(b->cfg, b->d_tdescs, b->nact, i, s));
        BCK(b, launch_forces_batch(b->cfg, b->d_tdescs, b->nact, i, s));
        BCK(b, launch_particle_kinematics_batch(b->cfg, b->d_tdescs, b->nact, i, s));
    }
    BCK(b, launch_advance_steps(b->d_ctls, (int)b->sims.size(), n, s));
    return MPM_OK;
}

int run_batch_graph(MpmBatch* b, int n, cudaStream_t s) {
    int r0 = prepare_tiles(b, s);
    if (r0 != MPM_OK) return r0;
    const int64_t key = (int64_t)n | ((int64_t)b->nact << 24) | ((int64_t)b->nemp << 44);
    auto it = b->graphs.find(key);
    if (it == b->graphs.end()) {
        cudaGraph_t g = nullptr;
        BCK(b, cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
        int r = launch_batch_steps(b, n, b->cap);
        cudaError_t e = cudaStreamEndCapture(b->cap, &g);
        if (r != MPM_OK) {
            if (g) cudaGraphDestroy(g);
            return r;
        }
        BCK(b, e);
        cudaGraphExec_t ex = nullptr;
        e = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        BCK(b, e);
        it = b->graphs.emplace(key, ex).first;
    }
    BCK(b, cudaGraphLaunch(it->second, s));
    return MPM_OK;
}

int check_ready(MpmBatch* b) {
    for (size_t i = 0; i < b->sims.size(); ++i) {
        MpmHandle* h = b->sims[i];
        if (!h->initialized || h->np <= 0)
            return bfail(b, MPM_ERR_STATE, "simulation %zu is not initialised with particles", i);
        if (h->has_trac != b->cfg.traction)
            return bfail(b, MPM_ERR_STATE, "simulation %zu changed its traction set-up", i);
    }
    return MPM_OK;
}

// Gather every simulation's control block into h_status and clear the status words.
int read_statuses(MpmBatch* b, cudaStream_t s) {
    const int n = (int)b->sims.size();
    BCK(b, launch_gather_status(b->d_ctls, n, b->d_status, s));
    BCK(b, cudaMemcpyAsync(b->h_status, b->d_status, sizeof(Control) * n, cudaMemcpyDeviceToHost, s));
    BCK(b, cudaStreamSynchronize(s));
    return MPM_OK;
}

// One block of B steps for every simulation (see the file comment).
int batch_block(MpmBatch* b, int B, cudaStream_t s) {
    const int n = (int)b->sims.size();
    if ((int)b->since_resort.size() != n) b->since_resort.assign(n, 0);
    for (int i = 0; i < n; ++i) {
        // a drifted simulation keeps its sort for resort_every - 1 more blocks
        // (its drifted cells take the gathering path); a two-cell drift
        // rolls the block back and replays it with re-sorts either way
        if (!b->sims[i]->needs_resort) {
            b->since_resort[i] = 0;
        } else if (++b->since_resort[i] >= b->resort_every) {
            BTRY(b, i, resort(b->sims[i], s));
            b->since_resort[i] = 0;
        }
    }
    std::vector<CopySeg> v;
    for (MpmHandle* h : b->sims) snapshot_segments(h, true, v);
    BTRY(b, 0, run_segments(b->sims[0], b->segbuf, v, s));
    std::vector<int64_t> step0(n);
    for (int i = 0; i < n; ++i) step0[i] = b->sims[i]->step;
    int r = run_batch_graph(b, B, s);
    if (r != MPM_OK) return r;
    for (MpmHandle* h : b->sims) {
        h->step += B;
        h->gen++;
    }
    r = read_statuses(b, s);
    if (r != MPM_OK) return r;
    for (int i = 0; i < n; ++i) {
        MpmHandle* h = b->sims[i];
        int st = b->h_status[i].status;
        // a two-cell drift corrupts the rest of the block: roll back first
        if (st & ST_DRIFT_VIOLATION) BTRY(b, i, replay_block(h, step0[i], B, st, s));
        else if (st & ST_OUT_OF_MESH)
            return bfail(b, MPM_ERR_OUT_OF_MESH, "simulation %d: a particle left the mesh", i);
        h->needs_resort = (st & ST_DRIFTED) != 0;
    }
    return MPM_OK;
}

int batch_steps(MpmBatch* b, int nsteps, cudaStream_t s) {
    while (nsteps > 0) {
        const int B = std::min(nsteps, b->block_steps);
        const int r = batch_block(b, B, s);
        if (r != MPM_OK) return r;
        nsteps -= B;
    }
    return MPM_OK;
}

// Save (or restore) the full state of every simulation in b->tune.
int tune_state(MpmBatch* b, bool save, cudaStream_t s) {
    const int n = (int)b->sims.size();
    if ((int)b->tune.size() != n) b->tune.resize(n);
    std::vector<CopySeg> v;
    for (int i = 0; i < n; ++i) {
        if (save) BTRY(b, i, checkpoint_alloc(b->sims[i], b->tune[i]));
        checkpoint_segments(b->sims[i], b->tune[i], save, v);
    }
    BTRY(b, 0, run_segments(b->sims[0], b->segbuf, v, s));
    BCK(b, cudaStreamSynchronize(s));
    return MPM_OK;
}

}  // namespace batch
}  // namespace mpm

using namespace mpm::batch;

extern "C" {

int mpm_batch_create(MpmHandle* const* sims, int n, MpmBatch** out) {
    if (!out || !sims || n < 1) return bfail(nullptr, MPM_ERR_INVALID, "need at least one simulation");
    *out = nullptr;
    std::set<MpmHandle*> seen;
    for (int i = 0; i < n; ++i) {
        MpmHandle* h = sims[i];
        if (!h) return bfail(nullptr, MPM_ERR_INVALID, "simulation %d is null", i);
        if (!seen.insert(h).second) return bfail(nullptr, MPM_ERR_INVALID, "simulation %d appears twice", i);
        if (!h->initialized || h->np <= 0)
            return bfail(nullptr, MPM_ERR_STATE, "simulation %d is not initialised with particles", i);
        if (h->ndim != 2)
            return bfail(nullptr, MPM_ERR_UNSUPPORTED, "batches hold Quadrilateral4Node simulations");
        if (h->device != sims[0]->device)
            return bfail(nullptr, MPM_ERR_INVALID, "simulations are on different devices");
        if (h->usl != sims[0]->usl || h->reinit != sims[0]->reinit || h->has_trac != sims[0]->has_trac)
            return bfail(nullptr, MPM_ERR_UNSUPPORTED,
                         "simulation %d: a batch needs one scheme, volume set-up and traction set-up", i);
    }
    MpmBatch* b = new MpmBatch();
    b->device = sims[0]->device;
    b->sims.assign(sims, sims + n);
    b->cfg.usl = sims[0]->usl;
    b->cfg.reinit = sims[0]->reinit;
    b->cfg.traction = sims[0]->has_trac;
    b->cfg.nk_ctas = sims[0]->nk_ctas;
    b->cfg.g2p_ctas = sims[0]->g2p_ctas;
    b->cfg.forces_lpc = sims[0]->forces_lpc;
    std::vector<int4> tiles;
    std::vector<const SimDev*> ds(n);
    std::vector<Control*> ctl(n);
    for (int i = 0; i < n; ++i) {
        const SimDev& S = sims[i]->hs;
        for (int ty = 0; ty < S.tiles_y; ++ty)
            for (int tx = 0; tx < S.tiles_x; ++tx) tiles.push_back(make_int4(i, tx, ty, 0));
        ds[i] = sims[i]->ds;
        ctl[i] = sims[i]->ctl;
    }
    b->ntiles = (int)tiles.size();
    auto bail = [&](const char* what, cudaError_t e) {
        bfail(nullptr, MPM_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
        mpm_batch_destroy(b);
        return e == cudaErrorMemoryAllocation ? MPM_ERR_NOMEM : MPM_ERR_CUDA;
    };
    cudaError_t e;
    if ((e = cudaMalloc(&b->d_sims, sizeof(SimDev*) * n)) != cudaSuccess) return bail("cudaMalloc", e);
    if ((e = cudaMalloc(&b->d_tdescs, sizeof(TileDesc) * tiles.size())) != cudaSuccess ||
        (e = cudaMalloc(&b->d_edescs, sizeof(TileDesc) * tiles.size())) != cudaSuccess ||
        (e = cudaMalloc(&b->d_act_list, sizeof(int4) * tiles.size())) != cudaSuccess ||
        (e = cudaMalloc(&b->d_emp_list, sizeof(int4) * tiles.size())) != cudaSuccess ||
        (e = cudaMalloc(&b->d_tflags, sizeof(int) * tiles.size())) != cudaSuccess ||
        (e = cudaMalloc(&b->d_tcounts, sizeof(int) * 2)) != cudaSuccess)
        return bail("cudaMalloc", e);
    if ((e = cudaMallocHost(&b->h_tcounts, sizeof(int) * 2)) != cudaSuccess) return bail("cudaMallocHost", e);
    if ((e = cudaMalloc(&b->d_ctls, sizeof(Control*) * n)) != cudaSuccess) return bail("cudaMalloc", e);
    if ((e = cudaMalloc(&b->d_tiles, sizeof(int4) * tiles.size())) != cudaSuccess) return bail("cudaMalloc", e);
    if ((e = cudaMalloc(&b->d_status, sizeof(Control) * n)) != cudaSuccess) return bail("cudaMalloc", e);
    if ((e = cudaMallocHost(&b->h_status, sizeof(Control) * n)) != cudaSuccess) return bail("cudaMallocHost", e);
    if ((e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking)) != cudaSuccess)
        return bail("cudaStreamCreate", e);
    if ((e = cudaMemcpy(b->d_sims, ds.data(), sizeof(SimDev*) * n, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(b->d_ctls, ctl.data(), sizeof(Control*) * n, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(b->d_tiles, tiles.data(), sizeof(int4) * tiles.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
        return bail("cudaMemcpy", e);
    *out = b;
    return MPM_OK;
}

int mpm_batch_destroy(MpmBatch* b) {
    if (!b) return MPM_OK;
    mpm::batch_adjoint_free(b);
    drop_batch_graphs(b);
    // (the autotuner's saved states belong to the handles, which free them)
    segbuf_free(b->segbuf);
    if (b->cap) cudaStreamDestroy(b->cap);
    cudaFree(b->d_sims);
    cudaFree(b->d_tdescs);
    cudaFree(b->d_edescs);
    cudaFree(b->d_act_list);
    cudaFree(b->d_emp_list);
    cudaFree(b->d_tflags);
    cudaFree(b->d_tcounts);
    if (b->h_tcounts) cudaFreeHost(b->h_tcounts);
    cudaFree(b->d_stage);
    cudaFree(b->d_ctls);
    cudaFree(b->d_tiles);
    cudaFree(b->d_status);
    if (b->h_status) cudaFreeHost(b->h_status);
    delete b;
    return MPM_OK;
}

const char* mpm_batch_last_error(const MpmBatch* b) {
    return b ? b->err.c_str() : g_batch_create_error.c_str();
}

int mpm_batch_size(const MpmBatch* b, int* n, int* ntiles) {
    if (!b) return MPM_ERR_INVALID;
    if (n) *n = (int)b->sims.size();
    if (ntiles) *ntiles = b->ntiles;
    return MPM_OK;
}

// ---------------------------------------------------------------------------
// Whole-batch state transfers: one host copy for every member, per-member
// gathers into storage order on the stream, one wait at the end.
// ---------------------------------------------------------------------------
static int batch_stage(MpmBatch* b, size_t bytes) {
    if (b->stage_bytes >= bytes) return MPM_OK;
    cudaFree(b->d_stage);
    b->d_stage = nullptr;
    b->stage_bytes = 0;
    BCK(b, cudaMalloc(&b->d_stage, bytes));
    b->stage_bytes = bytes;
    return MPM_OK;
}

static bool batch_writable(int field) {
    return field == MPM_FIELD_LOC || field == MPM_FIELD_VELOCITY || field == MPM_FIELD_STRESS ||
           field == MPM_FIELD_STRAIN || field == MPM_FIELD_DENSITY || field == MPM_FIELD_VSC;
}

int mpm_batch_write_field(MpmBatch* b, int field, const void* src, int on_device, void* stream) {
    if (!b || !src) return MPM_ERR_INVALID;
    if (!batch_writable(field))
        return bfail(b, MPM_ERR_INVALID, "field %d cannot be written for a whole batch", field);
    cudaStream_t s = S(stream);
    size_t total = 0;
    for (MpmHandle* h : b->sims) total += sizeof(float) * ncomp_of(h, field) * h->np;
    const char* d = static_cast<const char*>(src);
    if (!on_device) {
        int r = batch_stage(b, total);
        if (r != MPM_OK) return r;
        BCK(b, cudaMemcpyAsync(b->d_stage, src, total, cudaMemcpyHostToDevice, s));
        d = static_cast<const char*>(b->d_stage);
    }
    size_t off = 0;
    for (int i = 0; i < (int)b->sims.size(); ++i) {
        MpmHandle* h = b->sims[i];
        h->gen++;
        BTRY(b, i, write_float_field(h, field, reinterpret_cast<const float*>(d + off), s));
        off += sizeof(float) * ncomp_of(h, field) * h->np;
    }
    BCK(b, cudaStreamSynchronize(s));
    return MPM_OK;
}

int mpm_batch_read_field(MpmBatch* b, int field, void* dst, int on_device, void* stream) {
    if (!b || !dst) return MPM_ERR_INVALID;
    if (field < 0 || field >= MPM_FIELD_COUNT) return bfail(b, MPM_ERR_INVALID, "unknown field %d", field);
    cudaStream_t s = S(stream);
    size_t total = 0;
    for (MpmHandle* h : b->sims) total += sizeof(float) * ncomp_of(h, field) * h->np;
    char* d = static_cast<char*>(dst);
    if (!on_device) {
        int r = batch_stage(b, total);
        if (r != MPM_OK) return r;
        d = static_cast<char*>(b->d_stage);
    }
    size_t off = 0;
    for (int i = 0; i < (int)b->sims.size(); ++i) {
        MpmHandle* h = b->sims[i];
        BTRY(b, i, gather_field(h, field, d + off, s));
        off += sizeof(float) * ncomp_of(h, field) * h->np;
    }
    if (!on_device) BCK(b, cudaMemcpyAsync(dst, b->d_stage, total, cudaMemcpyDeviceToHost, s));
    BCK(b, cudaStreamSynchronize(s));
    return MPM_OK;
}

int mpm_batch_write_nodal_field(MpmBatch* b, int field, const float* src, int on_device, void* stream) {
    if (!b || !src) return MPM_ERR_INVALID;
    if (field != MPM_NODE_MASS && field != MPM_NODE_VELOCITY && field != MPM_NODE_ACCELERATION)
        return bfail(b, MPM_ERR_INVALID, "nodal field %d is not writable", field);
    cudaStream_t s = S(stream);
    const int nc = field == MPM_NODE_MASS ? 1 : 2;
    size_t total = 0;
    for (MpmHandle* h : b->sims) total += sizeof(float) * nc * h->nn;
    const char* d = reinterpret_cast<const char*>(src);
    if (!on_device) {
        int r = batch_stage(b, total);
        if (r != MPM_OK) return r;
        BCK(b, cudaMemcpyAsync(b->d_stage, src, total, cudaMemcpyHostToDevice, s));
        d = static_cast<const char*>(b->d_stage);
    }
    size_t off = 0;
    for (MpmHandle* h : b->sims) {
        h->gen++;
        const float* df = reinterpret_cast<const float*>(d + off);
        if (field == MPM_NODE_MASS)
            BCK(b, cudaMemcpyAsync(h->nm, df, sizeof(float) * h->nn, cudaMemcpyDeviceToDevice, s));
        else if (field == MPM_NODE_VELOCITY) BCK(b, launch_deinterleave2(df, h->nn, h->nvbx, h->nvby, s));
        else BCK(b, launch_deinterleave2(df, h->nn, h->nax, h->nay, s));
        off += sizeof(float) * nc * h->nn;
    }
    BCK(b, cudaStreamSynchronize(s));
    return MPM_OK;
}

int mpm_batch_restart(MpmBatch* b, void* stream) {
    if (!b) return MPM_ERR_INVALID;
    cudaStream_t s = S(stream);
    const int n = (int)b->sims.size();
    for (int i = 0; i < n; ++i) {
        MpmHandle* h = b->sims[i];
        h->gen++;
        BTRY(b, i, keep_parity_data(h, 0));
        h->step = 0;
        BCK(b, cudaMemsetAsync(h->ctl, 0, sizeof(Control), s));
        BTRY(b, i, resort(h, s));
        if (!h->reinit) BCK(b, launch_setup_volume(h->ds, (int)h->np, parity(h), s));
        h->initialized = true;
    }
    int r = read_statuses(b, s);
    if (r != MPM_OK) return r;
    for (int i = 0; i < n; ++i) {
        MpmHandle* h = b->sims[i];
        *h->h_ctl = b->h_status[i];
        int st = b->h_status[i].status;
        if (check_status(h, st) != MPM_OK) return from_sim(b, i, MPM_ERR_OUT_OF_MESH);
    }
    return MPM_OK;
}

int mpm_batch_set_block_steps(MpmBatch* b, int steps) {
    if (!b || steps < 1) return MPM_ERR_INVALID;
    b->block_steps = steps;
    return MPM_OK;
}

int mpm_batch_step(MpmBatch* b, int nsteps, void* stream) {
    if (!b) return MPM_ERR_INVALID;
    if (nsteps < 0) return bfail(b, MPM_ERR_INVALID, "nsteps must be >= 0");
    int r = check_ready(b);
    if (r != MPM_OK) return r;
    cudaStream_t s = S(stream);
    r = batch_steps(b, nsteps, s);
    if (r != MPM_OK) return r;
    BCK(b, cudaStreamSynchronize(s));
    return MPM_OK;
}

int mpm_batch_set_tuning(MpmBatch* b, const MpmTuning* t) {
    if (!b || !t) return MPM_ERR_INVALID;
    if (t->block_steps < 1 || t->resort_every < 1 || (t->nk_ctas != 2 && t->nk_ctas != 3) ||
        (t->g2p_ctas != 2 && t->g2p_ctas != 3) || t->forces_lpc < 0 || t->forces_lpc > 2)
        return bfail(b, MPM_ERR_INVALID, "tuning out of range (block_steps >= 1, resort_every >= 1, "
                                         "2 or 3 CTAs per SM, forces_lpc 0, 1 or 2)");
    if (t->nk_ctas != b->cfg.nk_ctas || t->g2p_ctas != b->cfg.g2p_ctas ||
        t->forces_lpc != b->cfg.forces_lpc) {
        b->cfg.nk_ctas = t->nk_ctas;
        b->cfg.g2p_ctas = t->g2p_ctas;
        b->cfg.forces_lpc = t->forces_lpc;
        drop_batch_graphs(b);   // the captured graphs hold the other builds
    }
    b->block_steps = t->block_steps;
    b->resort_every = t->resort_every;
    // the members' own steps and adjoints use the same builds
    for (MpmHandle* h : b->sims) {
        const int r = mpm_set_kernel_variant(h, t->nk_ctas, t->g2p_ctas, t->forces_lpc);
        if (r != MPM_OK) return r;
    }
    return MPM_OK;
}

int mpm_batch_get_tuning(const MpmBatch* b, MpmTuning* t) {
    if (!b || !t) return MPM_ERR_INVALID;
    t->block_steps = b->block_steps;
    t->resort_every = b->resort_every;
    t->nk_ctas = b->cfg.nk_ctas;
    t->g2p_ctas = b->cfg.g2p_ctas;
    t->forces_lpc = b->cfg.forces_lpc;
    t->ms_per_step = 0.0f;
    return MPM_OK;
}

namespace {

// Time trial_steps steps of the batch from the saved state with tuning t
// (the first pass captures the block graphs, the second is timed).
int time_tuning(MpmBatch* b, const MpmTuning& t, int trial_steps, cudaEvent_t e0, cudaEvent_t e1,
                cudaStream_t s, float* ms) {
    int r = mpm_batch_set_tuning(b, &t);
    for (int pass = 0; pass < 2 && r == MPM_OK; ++pass) {
        r = tune_state(b, false, s);
        if (r != MPM_OK) break;
        b->since_resort.assign(b->sims.size(), 0);
        if (cudaEventRecord(e0, s) != cudaSuccess) r = bfail(b, MPM_ERR_CUDA, "event record");
        if (r == MPM_OK) r = batch_steps(b, trial_steps, s);
        if (r == MPM_OK && cudaEventRecord(e1, s) != cudaSuccess) r = bfail(b, MPM_ERR_CUDA, "event record");
        if (r == MPM_OK && cudaEventSynchronize(e1) != cudaSuccess) r = bfail(b, MPM_ERR_CUDA, "event sync");
    }
    if (r == MPM_OK) cudaEventElapsedTime(ms, e0, e1);
    return r;
}

}  // namespace

int mpm_batch_autotune(MpmBatch* b, int trial_steps, MpmTuning* best_out, void* stream) {
    if (!b || trial_steps < 1) return MPM_ERR_INVALID;
    int r = check_ready(b);
    if (r != MPM_OK) return r;
    cudaStream_t s = S(stream);
    r = tune_state(b, true, s);
    if (r != MPM_OK) return r;
    cudaEvent_t e0, e1;
    BCK(b, cudaEventCreate(&e0));
    BCK(b, cudaEventCreate(&e1));
    // coordinate descent from the current tuning: kernel builds, then the
    // graph block length, then the re-sort cadence
    MpmTuning best;
    mpm_batch_get_tuning(b, &best);
    float best_ms = -1.0f;
    auto trial = [&](const MpmTuning& t) {
        float ms = 0.0f;
        if (r == MPM_OK) r = time_tuning(b, t, trial_steps, e0, e1, s, &ms);
        if (r == MPM_OK && (best_ms < 0.0f || ms < best_ms)) {
            best_ms = ms;
            best = t;
        }
    };
    trial(best);
    for (int nk : {3, 2})
        for (int g2p : {3, 2}) {
            MpmTuning t = best;
            t.nk_ctas = nk;
            t.g2p_ctas = g2p;
            if (t.nk_ctas != best.nk_ctas || t.g2p_ctas != best.g2p_ctas) trial(t);
        }
    {
        const int base_lpc = best.forces_lpc;
        for (int m : {0, 1, 2}) {
            MpmTuning t = best;
            t.forces_lpc = m;
            if (m != base_lpc) trial(t);
        }
    }
    const int base_block = best.block_steps;
    for (int c : {10, 25, 50, 100, 200}) {
        MpmTuning t = best;
        t.block_steps = c < trial_steps ? c : trial_steps;
        if (t.block_steps != base_block) trial(t);
    }
    for (int e : {2, 4}) {
        MpmTuning t = best;
        t.resort_every = e;
        if (t.block_steps * e <= trial_steps) trial(t);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const int r2 = r == MPM_OK ? mpm_batch_set_tuning(b, &best) : MPM_OK;
    const int r3 = tune_state(b, false, s);
    if (r != MPM_OK) return r;
    if (r2 != MPM_OK) return r2;
    if (r3 != MPM_OK) return r3;
    b->since_resort.assign(b->sims.size(), 0);
    best.ms_per_step = best_ms / (float)trial_steps;
    if (best_out) *best_out = best;
    return MPM_OK;
}

}  // extern "C"
