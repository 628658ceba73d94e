// C ABI of the GB300 explicit MPM step (declared in include/diffmpm_gb300.h).
//
// Host driver.  mpm_step advances in blocks of `block_steps` steps.  Each block
// is one CUDA graph of three launches per step over the active tiles (nodal
// kinematics, forces + nodal update, G2P), plus the empty tiles' node kernel
// when the handle launches those tiles apart.  Before a block the particles are re-sorted by cell if any
// particle changed cell during the previous block; the block's start state is
// snapshotted, and if a particle drifted two cells from its sort-cell inside
// the block (the cell gathers only look one cell away) the block is rolled back
// and replayed one step at a time with a re-sort before every step.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "mpm_handle.h"

using namespace mpm;

namespace {

thread_local std::string g_create_error;

}  // namespace

namespace mpm {
namespace host {

int fail(MpmHandle* h, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (h) h->err = buf;
    else g_create_error = buf;
    return code;
}

void dfree(MpmHandle* h, void* p) {
    if (!p) return;
    for (size_t i = 0; i < h->allocs.size(); ++i) {
        if (h->allocs[i] == p) {
            h->allocs.erase(h->allocs.begin() + i);
            break;
        }
    }
    cudaFree(p);
}

void drop_graphs(MpmHandle* h) {
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
    h->graphs.clear();
    h->graph_gen++;
}

int upload_desc(MpmHandle* h) {
    drop_graphs(h);
    CK(h, cudaMemcpy(h->ds, &h->hs, sizeof(SimDev), cudaMemcpyHostToDevice));
    return MPM_OK;
}

void bind_particles(MpmHandle* h) {
    PSet& p = h->ps[h->pcur];
    SimDev& s = h->hs;
    s.np = (int)h->np;
    s.x = p.x; s.y = p.y; s.vx = p.vx; s.vy = p.vy;
    for (int k = 0; k < 2; ++k) {
        s.sxx[k] = p.sxx[k]; s.syy[k] = p.syy[k]; s.szz[k] = p.szz[k]; s.sxy[k] = p.sxy[k];
        s.rho[k] = p.rho[k]; s.vsc[k] = p.vsc[k]; s.vol[k] = p.vol[k];
    }
    s.exx = p.exx; s.eyy = p.eyy; s.exy = p.exy;
    s.mass = p.mass;
    s.psize = p.psize;
    s.mat = p.mat;
    s.E = h->has_E ? p.E : nullptr;
    s.tr_fn = h->has_trac ? p.tr_fn : nullptr;
    s.tr_tau = h->has_trac ? p.tr_tau : nullptr;
    s.pvc = h->has_pvc ? p.pvc : nullptr;
    s.pvc_vel = h->d_pvc_vel;
    s.pid = p.pid;
    s.cstart = h->cstart[h->cs_cur];
    s.cflag = h->cflag;
}

int parity(const MpmHandle* h) { return (int)(h->step & 1); }

// All per-particle 4-byte arrays of a set that move with a re-sort (current parity
// for the ping-pong pairs), in a fixed order shared by the snapshot.
std::vector<float**> movable_f32(MpmHandle* h, PSet& p, bool for_snapshot) {
    const int par = parity(h);
    std::vector<float**> v = {&p.x, &p.y, &p.vx, &p.vy, &p.sxx[par], &p.syy[par], &p.szz[par],
                              &p.sxy[par], &p.exx, &p.eyy, &p.exy, &p.rho[par], &p.vsc[par]};
    if (!h->reinit) v.push_back(&p.vol[par]);
    if (!for_snapshot) {
        if (!h->reinit) {
            v.push_back(&p.mass);
            v.push_back(&p.psize);
        }
        if (h->has_E) v.push_back(&p.E);
        v.push_back(reinterpret_cast<float**>(&p.pid));
    }
    return v;
}

int ensure_stage(MpmHandle* h, size_t bytes) {
    if (h->stage_bytes >= bytes) return MPM_OK;
    dfree(h, h->stage);
    h->stage = nullptr;
    h->stage_bytes = 0;
    TRY(dalloc(h, reinterpret_cast<char**>(&h->stage), bytes));
    h->stage_bytes = bytes;
    return MPM_OK;
}

int sync(MpmHandle* h, cudaStream_t s) {
    CK(h, cudaStreamSynchronize(s));
    return MPM_OK;
}

int read_ctl(MpmHandle* h, cudaStream_t s) {
    CK(h, cudaMemcpyAsync(h->h_ctl, h->ctl, sizeof(Control), cudaMemcpyDeviceToHost, s));
    return sync(h, s);
}

int clear_status(MpmHandle* h, cudaStream_t s) {
    CK(h, cudaMemsetAsync(&h->ctl->status, 0, sizeof(int), s));
    return MPM_OK;
}

// Stable re-sort of the particles by current cell.
int resort(MpmHandle* h, cudaStream_t s) {
    if (h->np <= 0) {
        h->needs_resort = false;
        return MPM_OK;
    }
    const int np = (int)h->np, nb = h->ncell + 1;
    adjoint_note_resort(h);
    SortScratch& w = h->sw;
    CK(h, cudaMemsetAsync(w.count, 0, sizeof(int) * nb, s));
    CK(h, cudaMemsetAsync(w.cursor, 0, sizeof(int) * nb, s));
    CK(h, launch_resort_keys(h->ds, np, h->nx, h->ny, h->hx, h->hy, w, h->ctl, s));
    int* start = h->cstart[h->cs_cur ^ 1];
    CK(h, launch_exclusive_scan(w.count, start, nb, w.block_sums, s));
    CK(h, launch_resort_place(np, start, w, s));
    PSet& src = h->ps[h->pcur];
    PSet& dst = h->ps[h->pcur ^ 1];
    if (h->ndim == 1) CK(h, launch_line_segsort(nb, start, w.perm, src.pid, s));
    else CK(h, launch_resort_segsort(nb, start, w, s));
    std::vector<float**> a = movable_f32(h, src, false), b = movable_f32(h, dst, false);
    for (size_t i = 0; i < a.size(); ++i)
        CK(h, launch_gather_u32(reinterpret_cast<const uint32_t*>(*a[i]),
                                reinterpret_cast<uint32_t*>(*b[i]), w.perm, np, s));
    CK(h, launch_gather_u8(src.mat, dst.mat, w.perm, np, s));
    if (h->has_pvc) CK(h, launch_gather_pair_u8(src.pvc, dst.pvc, w.perm, np, s));
    if (h->has_trac) {
        CK(h, launch_gather_pair_u8(reinterpret_cast<const uint8_t*>(src.tr_fn),
                                    reinterpret_cast<uint8_t*>(dst.tr_fn), w.perm, np, s));
        CK(h, launch_gather_pair_u32(reinterpret_cast<const uint32_t*>(src.tr_tau),
                                     reinterpret_cast<uint32_t*>(dst.tr_tau), w.perm, np, s));
    }
    h->pcur ^= 1;
    h->cs_cur ^= 1;
    CK(h, cudaMemsetAsync(h->cflag, 0, h->ncell, s));
    if (h->ndim == 1) CK(h, launch_line_eid(start, h->nx, h->line_eid, s));
    bind_particles(h);
    drop_graphs(h);   // the step graphs hold the descriptor by value
    CK(h, cudaMemcpyAsync(h->ds, &h->hs, sizeof(SimDev), cudaMemcpyHostToDevice, s));
    h->needs_resort = false;
    h->resorts++;
    return MPM_OK;
}

int take_snapshot(MpmHandle* h, cudaStream_t s) {
    if (h->snap_f.size() != movable_f32(h, h->ps[h->pcur], true).size())
        return fail(h, MPM_ERR_STATE, "snapshot layout mismatch");
    std::vector<CopySeg> v;
    snapshot_segments(h, true, v);
    return run_segments(h, h->segbuf, v, s);
}

int restore_snapshot(MpmHandle* h, int64_t step0, cudaStream_t s) {
    h->step = step0;
    std::vector<CopySeg> v;
    snapshot_segments(h, false, v);
    TRY(run_segments(h, h->segbuf, v, s));
    TRY(clear_status(h, s));
    return sync(h, s);
}

StepConfig step_config(const MpmHandle* h) {
    StepConfig c;
    c.usl = h->usl;
    c.reinit = h->reinit;
    c.traction = h->has_trac;
    c.nk_ctas = h->nk_ctas;
    c.g2p_ctas = h->g2p_ctas;
    c.forces_lpc = h->forces_lpc;
    return c;
}

// Split the tiles into active and empty ones for the current sort (see
// launch_classify_tiles); every launched sequence of steps starts with it.
int classify_tiles(MpmHandle* h, cudaStream_t s) {
    CK(h, launch_classify_tiles(h->hs, h->dtiles, h->ntiles, h->d_tile_flags, h->d_active, h->d_empty,
                                h->d_tile_counts, s));
    CK(h, cudaMemcpyAsync(h->h_tile_counts, h->d_tile_counts, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(h, cudaStreamSynchronize(s));
    if (h->h_tile_counts[1] < h->empty_split_min) {
        // too few empty tiles to pay for a launch of their own: the step
        // kernels take every tile (an empty one costs a CTA that only
        // updates its nodes, in a grid that is often under one wave)
        h->step_tiles = h->dtiles;
        h->nact = h->ntiles;
        h->nemp = 0;
    } else {
        h->step_tiles = h->d_active;
        h->nact = tile_grid(h->h_tile_counts[0], h->ntiles);
        h->nemp = tile_grid(h->h_tile_counts[1], h->ntiles);
    }
    return MPM_OK;
}

// Graph-cache key of a step sequence: its length and the grids it launches.
int64_t seq_key(const MpmHandle* h, int n) {
    return (int64_t)n | ((int64_t)h->nact << 24) | ((int64_t)h->nemp << 44);
}

// One phase of step (ctl->step + k) over the active tiles (the empty tiles'
// nodes are updated with the nodal kinematics); phase 2 ends the step, whose
// counter the caller advances.
int launch_phase(MpmHandle* h, int phase, int k, cudaStream_t s) {
    const StepConfig c = step_config(h);
    cudaError_t e = cudaSuccess;
    if (phase == 0) {
        CK(h, launch_empty_nodes(h->hs, h->d_empty, h->nemp, h->ctl, k, s));
        e = launch_nodal_kinematics(c, h->hs, h->step_tiles, h->nact, h->ctl, k, s);
    } else if (phase == 1) {
        e = launch_forces(c, h->hs, h->step_tiles, h->nact, h->ctl, k, s);
    } else {
        e = launch_particle_kinematics(c, h->hs, h->step_tiles, h->nact, h->ctl, k, s);
    }
    CK(h, e);
    return MPM_OK;
}

int launch_steps(MpmHandle* h, int n, cudaStream_t s) {
    for (int i = 0; i < n; ++i)
        for (int p = 0; p < 3; ++p) TRY(launch_phase(h, p, i, s));
    CK(h, launch_advance_step(h->ctl, n, s));
    return MPM_OK;
}



int run_graph(MpmHandle* h, int n, cudaStream_t s) {
    if (h->graphs_trac != h->has_trac) {
        drop_graphs(h);
        h->graphs_trac = h->has_trac;
    }
    TRY(classify_tiles(h, s));
    const int64_t key = seq_key(h, n);
    auto it = h->graphs.find(key);
    if (it == h->graphs.end()) {
        cudaGraph_t g = nullptr;
        CK(h, cudaStreamBeginCapture(h->cap, cudaStreamCaptureModeThreadLocal));
        int r = launch_steps(h, n, h->cap);
        cudaError_t e = cudaStreamEndCapture(h->cap, &g);
        if (r != MPM_OK) {
            if (g) cudaGraphDestroy(g);
            return r;
        }
        CK(h, e);
        cudaGraphExec_t ex = nullptr;
        e = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        CK(h, e);
        it = h->graphs.emplace(key, ex).first;
    }
    CK(h, cudaGraphLaunch(it->second, s));
    return MPM_OK;
}

int check_status(MpmHandle* h, int& st) {
    st = h->h_ctl->status;
    if (st & ST_OUT_OF_MESH)
        return fail(h, MPM_ERR_OUT_OF_MESH,
                    "a particle left the mesh (the reference would give it a wrapped element id)");
    return MPM_OK;
}

int alloc_particles(MpmHandle* h, int64_t n) {
    // the step kernels stage particle rows in 16-byte pieces, which may read
    // up to 3 slots past the last particle: the float arrays hold a multiple
    // of 4 slots
    const int64_t n4 = (n + 3) & ~int64_t(3);
    for (int k = 0; k < 2; ++k) {
        PSet& p = h->ps[k];
        float** f32[] = {&p.x, &p.y, &p.vx, &p.vy, &p.sxx[0], &p.sxx[1], &p.syy[0], &p.syy[1],
                         &p.szz[0], &p.szz[1], &p.sxy[0], &p.sxy[1], &p.exx, &p.eyy, &p.exy,
                         &p.rho[0], &p.rho[1], &p.vsc[0], &p.vsc[1]};
        for (float** f : f32) TRY(dalloc(h, f, n4));
        if (!h->reinit) {
            TRY(dalloc(h, &p.mass, n4));
            TRY(dalloc(h, &p.psize, n4));
        }
        if (!h->reinit || h->ndim == 1) {   // 1-D keeps the updated volume for its forces kernel
            TRY(dalloc(h, &p.vol[0], n4));
            TRY(dalloc(h, &p.vol[1], n4));
        }
        TRY(dalloc(h, &p.mat, n));
        TRY(dalloc(h, &p.pid, n));
    }
    TRY(dalloc(h, &h->passive, 5 * n));
    TRY(dalloc(h, &h->sw.key, n));
    TRY(dalloc(h, &h->sw.perm, n));
    if (h->ndim == 1) TRY(dalloc(h, &h->line_eid, n));
    const size_t nsnap = movable_f32(h, h->ps[0], true).size();
    h->snap_f.assign(nsnap, nullptr);
    for (size_t i = 0; i < nsnap; ++i) TRY(dalloc(h, &h->snap_f[i], n));
    return MPM_OK;
}

void free_particles(MpmHandle* h) {
    for (int k = 0; k < 2; ++k) {
        PSet& p = h->ps[k];
        void* ptrs[] = {p.x, p.y, p.vx, p.vy, p.sxx[0], p.sxx[1], p.syy[0], p.syy[1], p.szz[0],
                        p.szz[1], p.sxy[0], p.sxy[1], p.exx, p.eyy, p.exy, p.rho[0], p.rho[1],
                        p.vsc[0], p.vsc[1], p.vol[0], p.vol[1], p.mass, p.psize, p.E, p.tr_tau,
                        p.mat, p.tr_fn, p.pvc, p.pid};
        for (void* q : ptrs) dfree(h, q);
        p = PSet{};
    }
    dfree(h, h->passive);
    h->passive = nullptr;
    dfree(h, h->sw.key);
    dfree(h, h->sw.perm);
    h->sw.key = h->sw.perm = nullptr;
    dfree(h, h->line_eid);
    h->line_eid = nullptr;
    for (float* f : h->snap_f) dfree(h, f);
    h->snap_f.clear();
    h->np = -1;
    h->has_trac = h->has_E = h->has_pvc = false;
}

// Bring device data of `bytes` at `src` into device memory (staging host data).
int to_device(MpmHandle* h, const void* src, size_t bytes, int on_device, cudaStream_t s,
              const void** dsrc) {
    if (on_device) {
        *dsrc = src;
        return MPM_OK;
    }
    TRY(ensure_stage(h, bytes));
    CK(h, cudaMemcpyAsync(h->stage, src, bytes, cudaMemcpyHostToDevice, s));
    *dsrc = h->stage;
    return MPM_OK;
}

int set_ptr_table(MpmHandle* h, const std::vector<float*>& ptrs, cudaStream_t s) {
    CK(h, cudaMemcpyAsync(h->d_ptrs, ptrs.data(), sizeof(float*) * ptrs.size(), cudaMemcpyHostToDevice, s));
    return MPM_OK;
}

int fill(MpmHandle* h, float* p, float v, int64_t n, cudaStream_t s) {
    std::vector<float> tmp((size_t)n, v);
    CK(h, cudaMemcpyAsync(p, tmp.data(), sizeof(float) * n, cudaMemcpyHostToDevice, s));
    return sync(h, s);
}

int ncomp_of(const MpmHandle* h, int field) {
    switch (field) {
        case MPM_FIELD_LOC:
        case MPM_FIELD_VELOCITY:
        case MPM_FIELD_MOMENTUM:
            return h->ndim;
        case MPM_FIELD_STRESS:
        case MPM_FIELD_STRAIN:
            return 6;
        default:
            return 1;
    }
}

// Storage-order component pointers of a float field (null = passive component).
std::vector<float*> comps(MpmHandle* h, int field) {
    PSet& p = h->ps[h->pcur];
    const int par = parity(h);
    switch (field) {
        case MPM_FIELD_LOC: return h->ndim == 1 ? std::vector<float*>{p.x} : std::vector<float*>{p.x, p.y};
        case MPM_FIELD_VELOCITY: return h->ndim == 1 ? std::vector<float*>{p.vx} : std::vector<float*>{p.vx, p.vy};
        case MPM_FIELD_STRESS: return {p.sxx[par], p.syy[par], p.szz[par], p.sxy[par], nullptr, nullptr};
        case MPM_FIELD_STRAIN: return {p.exx, p.eyy, nullptr, p.exy, nullptr, nullptr};
        case MPM_FIELD_DENSITY: return {p.rho[par]};
        case MPM_FIELD_VSC: return {p.vsc[par]};
        case MPM_FIELD_YOUNGS_MODULUS: return {p.E};
        case MPM_FIELD_VOLUME: return {p.vol[par]};
        case MPM_FIELD_MASS: return {p.mass};
        default: return {};
    }
}

// passive components: (field comp) -> slot in the 5-wide original-order array
int passive_slot(int field, int c) {
    if (field == MPM_FIELD_STRESS && c == 4) return 0;
    if (field == MPM_FIELD_STRESS && c == 5) return 1;
    if (field == MPM_FIELD_STRAIN && c == 2) return 2;
    if (field == MPM_FIELD_STRAIN && c == 4) return 3;
    if (field == MPM_FIELD_STRAIN && c == 5) return 4;
    return -1;
}

int copy_passive(MpmHandle* h, int field, float* aos, bool to_aos, cudaStream_t s) {
    for (int c = 0; c < 6; ++c) {
        const int slot = passive_slot(field, c);
        if (slot < 0) continue;
        float* pas = h->passive + slot;
        if (to_aos)
            CK(h, cudaMemcpy2DAsync(aos + c, 6 * sizeof(float), pas, 5 * sizeof(float), sizeof(float),
                                    h->np, cudaMemcpyDeviceToDevice, s));
        else
            CK(h, cudaMemcpy2DAsync(pas, 5 * sizeof(float), aos + c, 6 * sizeof(float), sizeof(float),
                                    h->np, cudaMemcpyDeviceToDevice, s));
    }
    return MPM_OK;
}

// Roll the block that started at step0 back to its snapshot and replay its B
// steps one at a time, re-sorting after every step that left a particle
// outside its sort-cell; `st` gets the last status.  A particle that leaves
// the mesh during the replay is an error; so is one that crosses two cells in
// a single step (the replay starts every step with drift at most one cell).
int replay_block(MpmHandle* h, int64_t step0, int B, int& st, cudaStream_t s) {
    h->rollbacks++;
    TRY(restore_snapshot(h, step0, s));
    st = 0;
    for (int i = 0; i < B; ++i) {
        if (st & ST_DRIFTED) TRY(resort(h, s));
        TRY(classify_tiles(h, s));
        TRY(launch_steps(h, 1, s));
        h->step++;
        TRY(read_ctl(h, s));
        TRY(check_status(h, st));
        if (st & ST_DRIFT_VIOLATION)
            return fail(h, MPM_ERR_CFL, "a particle crossed more than one cell in one step (step %lld)",
                        (long long)h->step - 1);
        TRY(clear_status(h, s));
    }
    return MPM_OK;
}

}  // namespace host
}  // namespace mpm

using namespace mpm::host;

void mpm::set_thread_error(const std::string& msg) { g_create_error = msg; }

extern "C" {

int mpm_abi_version(void) { return MPM_ABI_VERSION; }

const char* mpm_last_error(const MpmHandle* h) {
    return h ? h->err.c_str() : g_create_error.c_str();
}

int mpm_create(const MpmDesc* d, MpmHandle** out) {
    if (!d || !out) return fail(nullptr, MPM_ERR_INVALID, "null argument");
    *out = nullptr;
    if (d->ndim != 1 && d->ndim != 2)
        return fail(nullptr, MPM_ERR_UNSUPPORTED, "ndim=%d: Linear1D (1) and Quadrilateral4Node (2) only", d->ndim);
    const bool line = d->ndim == 1;
    if (d->nelements[0] < 1 || (!line && d->nelements[1] < 1))
        return fail(nullptr, MPM_ERR_INVALID, "nelements must be positive");
    const int64_t nn64 = line ? (int64_t)d->nelements[0] + 1
                              : (int64_t)(d->nelements[0] + 1) * (d->nelements[1] + 1);
    if (nn64 > (int64_t)1 << 30) return fail(nullptr, MPM_ERR_INVALID, "mesh too large");
    if (!(d->el_len[0] > 0) || (!line && !(d->el_len[1] > 0)))
        return fail(nullptr, MPM_ERR_INVALID, "element lengths must be positive");
    if (d->scheme != MPM_USF && d->scheme != MPM_USL)
        return fail(nullptr, MPM_ERR_INVALID, "Please select scheme from ('usf', 'usl'). Found %d", d->scheme);
    if (d->n_materials < 1 || d->n_materials > 255 || !d->materials)
        return fail(nullptr, MPM_ERR_INVALID, "need 1..255 materials");

    MpmHandle* h = new MpmHandle();
    cudaGetDevice(&h->device);
    // a 1-D mesh sorts its particles as one row of cells (y = 0, hy = 1)
    h->ndim = d->ndim;
    h->nx = d->nelements[0];
    h->ny = line ? 1 : d->nelements[1];
    h->hx = (float)d->el_len[0];
    h->hy = line ? 1.0f : (float)d->el_len[1];
    h->dt = (float)d->dt;
    h->gx = (float)d->gravity[0];
    h->gy = (float)d->gravity[1];
    h->usl = d->scheme == MPM_USL;
    // the forces kernel's lane-per-cell path is the faster one when it carries
    // no stress update (USL: 1024^2 scale-up 51 -> 38 us), the row path when
    // it does (USF: 68 vs 82 us)
    h->forces_lpc = h->usl ? 1 : 0;
    h->reinit = d->reinit_each_step != 0;
    h->velocity_update = d->velocity_update ? 1 : 0;
    h->vol_el = element_volume(h->hx, h->hy);
    h->nn = (int)nn64;
    h->ncell = h->nx * h->ny;
    auto bail = [&](int r) {
        mpm_destroy(h);
        return r;
    };
    auto failc = [&](int code, const char* msg) {
        g_create_error = msg;
        mpm_destroy(h);
        return code;
    };

    // materials (diffmpm/material.py:54-131); coefficients in float64, stored float32
    for (int i = 0; i < d->n_materials; ++i) {
        const MpmMaterial& m = d->materials[i];
        MatDev md{};
        md.type = m.type;
        md.density = (float)m.density;
        if (m.type == MPM_LINEAR_ELASTIC) {
            const double E = m.youngs_modulus, nu = m.poisson_ratio;
            const double K = E / (3 * (1 - 2 * nu));
            const double G = E / (2 * (1 + nu));
            md.a1 = (float)(K + (4 * G / 3));
            md.a2 = (float)(K - (2 * G / 3));
            md.G = (float)G;
            const double Ku = 1.0 / (3 * (1 - 2 * nu)), Gu = 1.0 / (2 * (1 + nu));
            md.c1 = (float)(Ku + 4 * Gu / 3);
            md.c2 = (float)(Ku - 2 * Gu / 3);
            md.c3 = (float)Gu;
        } else if (m.type == MPM_SIMPLE) {
            md.E = (float)m.E;
        } else if (m.type == MPM_NEWTONIAN) {
            md.K = (float)m.bulk_modulus;
            md.mu = (float)m.dynamic_viscosity;
            md.twomu = (float)(2.0 * m.dynamic_viscosity);
        } else {
            return failc(MPM_ERR_INVALID, "unknown material type");
        }
        h->mats.push_back(md);
    }
    h->nmat = d->n_materials;

    // constraint codes per node (diffmpm/constraint.py:29-44): last entry wins
    std::vector<uint16_t> code((size_t)h->nn, 0);
    std::vector<float> vel;
    for (int i = 0; i < d->n_constraints; ++i) {
        const int n = d->constraint_node[i], dir = d->constraint_dir[i];
        if (n < 0 || n >= h->nn) return failc(MPM_ERR_INVALID, "constraint node id out of range");
        if (dir != 0 && dir != 1) return failc(MPM_ERR_INVALID, "constraint dir must be 0 or 1");
        if (line && dir != 0) return failc(MPM_ERR_INVALID, "constraint dir must be 0 in 1-D");
        const float v = (float)d->constraint_velocity[i];
        int slot = -1;
        for (size_t k = 0; k < vel.size(); ++k)
            if (std::memcmp(&vel[k], &v, sizeof v) == 0) slot = (int)k;
        if (slot < 0) {
            if (vel.size() >= 255) return failc(MPM_ERR_UNSUPPORTED, "more than 255 distinct constraint velocities");
            vel.push_back(v);
            slot = (int)vel.size() - 1;
        }
        if (dir == 0) code[n] = (uint16_t)((code[n] & 0xff00) | (slot + 1));
        else code[n] = (uint16_t)((code[n] & 0x00ff) | ((slot + 1) << 8));
    }

    // time functions (diffmpm/functions.py:33-49)
    std::vector<int> fn_off(1, 0);
    std::vector<float> fx, fy;
    for (int k = 0; k < d->n_functions; ++k) {
        const int np = d->function_npoints[k];
        if (np < 1) return failc(MPM_ERR_INVALID, "a time function needs at least one point");
        for (int j = 0; j < np; ++j) {
            fx.push_back((float)d->function_x[fn_off.back() + j]);
            fy.push_back((float)d->function_y[fn_off.back() + j]);
        }
        fn_off.push_back(fn_off.back() + np);
    }
    h->nfn = d->n_functions;

    // concentrated nodal forces as CSR per node, list order kept within a node
    std::vector<int> cnf_ptr;
    std::vector<int8_t> cnf_dir, cnf_fn;
    std::vector<float> cnf_val;
    if (d->n_nodal_forces > 0) {
        cnf_ptr.assign((size_t)h->nn + 1, 0);
        for (int i = 0; i < d->n_nodal_forces; ++i) {
            const int n = d->nodal_force_node[i];
            if (n < 0 || n >= h->nn) return failc(MPM_ERR_INVALID, "nodal force node id out of range");
            if (d->nodal_force_dir[i] != 0 && d->nodal_force_dir[i] != (line ? 0 : 1))
                return failc(MPM_ERR_INVALID, line ? "nodal force dir must be 0 in 1-D"
                                                   : "nodal force dir must be 0 or 1");
            const int f = d->nodal_force_function[i];
            if (f < -1 || f >= d->n_functions) return failc(MPM_ERR_INVALID, "nodal force function out of range");
            cnf_ptr[n + 1]++;
        }
        for (int n = 0; n < h->nn; ++n) cnf_ptr[n + 1] += cnf_ptr[n];
        cnf_dir.resize(d->n_nodal_forces);
        cnf_fn.resize(d->n_nodal_forces);
        cnf_val.resize(d->n_nodal_forces);
        std::vector<int> cur(cnf_ptr.begin(), cnf_ptr.end() - 1);
        for (int i = 0; i < d->n_nodal_forces; ++i) {
            const int k = cur[d->nodal_force_node[i]]++;
            cnf_dir[k] = (int8_t)d->nodal_force_dir[i];
            cnf_fn[k] = (int8_t)(d->nodal_force_function[i] < 0 ? 1 : d->nodal_force_function[i] + 2);
            cnf_val[k] = (float)d->nodal_force_value[i];
        }
    }
    if (h->nfn > 120) return failc(MPM_ERR_UNSUPPORTED, "at most 120 time functions");

    // device allocations
    int r = MPM_OK;
#define A(p, n) if ((r = dalloc(h, p, n)) != MPM_OK) { g_create_error = h->err; return bail(r); }
    A(&h->d_mats, h->mats.size());
    A(&h->d_cons_vel, vel.size() + 1);
    A(&h->d_ncons, (size_t)h->nn);
    A(&h->d_fn_off, fn_off.size());
    A(&h->d_fn_x, fx.size() + 1);
    A(&h->d_fn_y, fy.size() + 1);
    if (!cnf_ptr.empty()) {
        A(&h->d_cnf_ptr, cnf_ptr.size());
        A(&h->d_cnf_dir, cnf_dir.size());
        A(&h->d_cnf_fn, cnf_fn.size());
        A(&h->d_cnf_val, cnf_val.size());
    }
    A(&h->nm, (size_t)h->nn);
    A(&h->nvax, (size_t)h->nn);
    A(&h->nvay, (size_t)h->nn);
    A(&h->nvbx, (size_t)h->nn);
    A(&h->nvby, (size_t)h->nn);
    A(&h->nax, (size_t)h->nn);
    A(&h->nay, (size_t)h->nn);
    A(&h->cstart[0], (size_t)h->ncell + 2);
    A(&h->cstart[1], (size_t)h->ncell + 2);
    A(&h->cflag, (size_t)h->ncell);
    A(&h->sw.count, (size_t)h->ncell + 1);
    A(&h->sw.cursor, (size_t)h->ncell + 1);
    A(&h->sw.block_sums, (size_t)(h->ncell + 2) / 1024 + 3);
    A(&h->snap_cflag, (size_t)h->ncell);
    A(&h->snap_nvbx, (size_t)h->nn);
    A(&h->snap_nvby, (size_t)h->nn);
    A(&h->snap_ctl, 1);
    A(&h->ds, 1);
    A(&h->ctl, 1);
    A(&h->d_ptrs, 16);
#undef A
    cudaError_t e = cudaMallocHost(&h->h_ctl, sizeof(Control));
    if (e == cudaSuccess) e = cudaMallocHost(&h->h_tile_counts, 2 * sizeof(int));
    if (e != cudaSuccess) return failc(MPM_ERR_NOMEM, "cudaMallocHost failed");
    e = cudaStreamCreateWithFlags(&h->cap, cudaStreamNonBlocking);
    if (e != cudaSuccess) return failc(MPM_ERR_CUDA, "cudaStreamCreate failed");

    auto up = [&](void* dst, const void* src, size_t bytes) {
        if (bytes && cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess) r = MPM_ERR_CUDA;
    };
    up(h->d_mats, h->mats.data(), sizeof(MatDev) * h->mats.size());
    up(h->d_cons_vel, vel.data(), sizeof(float) * vel.size());
    up(h->d_ncons, code.data(), sizeof(uint16_t) * code.size());
    up(h->d_fn_off, fn_off.data(), sizeof(int) * fn_off.size());
    up(h->d_fn_x, fx.data(), sizeof(float) * fx.size());
    up(h->d_fn_y, fy.data(), sizeof(float) * fy.size());
    if (!cnf_ptr.empty()) {
        up(h->d_cnf_ptr, cnf_ptr.data(), sizeof(int) * cnf_ptr.size());
        up(h->d_cnf_dir, cnf_dir.data(), cnf_dir.size());
        up(h->d_cnf_fn, cnf_fn.data(), cnf_fn.size());
        up(h->d_cnf_val, cnf_val.data(), sizeof(float) * cnf_val.size());
    }
    if (r != MPM_OK) return failc(r, "upload of the simulation tables failed");
    // nodal state at Nodes.__init__ (diffmpm/node.py:64-71): mass 1, the rest 0
    std::vector<float> ones((size_t)h->nn, 1.0f);
    up(h->nm, ones.data(), sizeof(float) * h->nn);
    for (float* p : {h->nvax, h->nvay, h->nvbx, h->nvby, h->nax, h->nay})
        if (cudaMemset(p, 0, sizeof(float) * h->nn) != cudaSuccess) r = MPM_ERR_CUDA;
    if (cudaMemset(h->cflag, 0, h->ncell) != cudaSuccess) r = MPM_ERR_CUDA;
    Control c{};
    up(h->ctl, &c, sizeof c);
    if (r != MPM_OK) return failc(r, "initialisation of the nodal state failed");

    // tiles
    std::vector<int4> tiles;
    const int tx = (h->nx + 1 + TILE_NX - 1) / TILE_NX, ty = (h->ny + 1 + TILE_NY - 1) / TILE_NY;
    for (int j = 0; j < ty; ++j)
        for (int i = 0; i < tx; ++i) tiles.push_back(make_int4(0, i, j, 0));
    h->ntiles = (int)tiles.size();
    if (dalloc(h, &h->dtiles, tiles.size()) != MPM_OK) {
        g_create_error = h->err;
        return bail(MPM_ERR_NOMEM);
    }
    up(h->dtiles, tiles.data(), sizeof(int4) * tiles.size());
    if (dalloc(h, &h->d_active, tiles.size()) != MPM_OK || dalloc(h, &h->d_empty, tiles.size()) != MPM_OK ||
        dalloc(h, &h->d_tile_flags, tiles.size()) != MPM_OK || dalloc(h, &h->d_tile_counts, 2) != MPM_OK) {
        g_create_error = h->err;
        return bail(MPM_ERR_NOMEM);
    }
    {
        // until the first classification: every tile active, none empty
        std::vector<int4> none(tiles.size(), make_int4(-1, 0, 0, 0));
        up(h->d_active, tiles.data(), sizeof(int4) * tiles.size());
        up(h->d_empty, none.data(), sizeof(int4) * tiles.size());
        h->nact = (int)tiles.size();
        h->nemp = 0;
        h->step_tiles = h->d_active;
    }
    if (r != MPM_OK) return failc(r, "tile upload failed");

    SimDev& s = h->hs;
    s.nx = h->nx; s.ny = h->ny; s.hx = h->hx; s.hy = h->hy; s.vol_el = h->vol_el; s.dt = h->dt;
    s.gx = h->gx; s.gy = h->gy; s.tiles_x = tx; s.tiles_y = ty; s.np = 0;
    s.velocity_update = h->velocity_update;
    s.nm = h->nm; s.nvax = h->nvax; s.nvay = h->nvay; s.nvbx = h->nvbx; s.nvby = h->nvby;
    s.nax = h->nax; s.nay = h->nay; s.ncons = h->d_ncons; s.cons_vel = h->d_cons_vel;
    s.cnf_ptr = h->d_cnf_ptr; s.cnf_dir = h->d_cnf_dir; s.cnf_val = h->d_cnf_val; s.cnf_fn = h->d_cnf_fn;
    s.nfn = h->nfn; s.fn_off = h->d_fn_off; s.fn_x = h->d_fn_x; s.fn_y = h->d_fn_y;
    s.nmat = h->nmat; s.mats = h->d_mats;
    s.cstart = h->cstart[0]; s.cflag = h->cflag;
    if (upload_desc(h) != MPM_OK) {
        g_create_error = h->err;
        return bail(MPM_ERR_CUDA);
    }
    *out = h;
    return MPM_OK;
}

int mpm_destroy(MpmHandle* h) {
    if (!h) return MPM_OK;
    mpm::adjoint_free(h);
    mpm::line_adjoint_free(h);
    segbuf_free(h->segbuf);
    drop_graphs(h);
    if (h->cap) cudaStreamDestroy(h->cap);
    for (cudaEvent_t& e : h->out_ev)
        if (e) cudaEventDestroy(e);
    for (void* p : h->allocs) cudaFree(p);
    h->allocs.clear();
    if (h->h_ctl) cudaFreeHost(h->h_ctl);
    if (h->h_tile_counts) cudaFreeHost(h->h_tile_counts);
    delete h;
    return MPM_OK;
}

int mpm_set_particles(MpmHandle* h, int64_t n, const float* loc, const int32_t* material_id,
                      int on_device, void* stream) {
    if (!h) return MPM_ERR_INVALID;
    h->gen++;
    if (n < 0 || n > ((int64_t)1 << 31) - 1) return fail(h, MPM_ERR_INVALID, "particle count out of range");
    if (n > 0 && !loc) return fail(h, MPM_ERR_INVALID, "loc is null");
    cudaStream_t s = S(stream);
    TRY(sync(h, s));
    if (h->np != n) {
        free_particles(h);
        drop_graphs(h);
        if (n > 0) TRY(alloc_particles(h, n));
        h->np = n;
    }
    h->has_trac = false;
    h->has_E = false;
    h->has_pvc = false;
    h->pcur = 0;
    h->cs_cur = 0;
    h->step = 0;
    h->initialized = false;
    PSet& p = h->ps[0];
    bind_particles(h);
    TRY(upload_desc(h));
    Control c{};
    *h->h_ctl = c;
    CK(h, cudaMemcpy(h->ctl, h->h_ctl, sizeof(Control), cudaMemcpyHostToDevice));
    if (n == 0) return MPM_OK;
    // identity storage order
    std::vector<int> ident((size_t)n);
    for (int64_t i = 0; i < n; ++i) ident[i] = (int)i;
    CK(h, cudaMemcpy(p.pid, ident.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    // materials and the reference's initial values (diffmpm/particle.py:53-71)
    std::vector<int32_t> mids((size_t)n, 0);
    if (material_id) {
        if (on_device) CK(h, cudaMemcpy(mids.data(), material_id, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
        else std::memcpy(mids.data(), material_id, sizeof(int32_t) * n);
    }
    std::vector<uint8_t> m8((size_t)n);
    std::vector<float> dens((size_t)n);
    for (int64_t i = 0; i < n; ++i) {
        if (mids[i] < 0 || mids[i] >= h->nmat) return fail(h, MPM_ERR_INVALID, "material id %d out of range", mids[i]);
        m8[i] = (uint8_t)mids[i];
        dens[i] = 1.0f * h->mats[mids[i]].density;
    }
    CK(h, cudaMemcpy(p.mat, m8.data(), n, cudaMemcpyHostToDevice));
    for (int k = 0; k < 2; ++k) CK(h, cudaMemcpy(p.rho[k], dens.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
    float* zero[] = {p.y, p.vx, p.vy, p.sxx[0], p.sxx[1], p.syy[0], p.syy[1], p.szz[0], p.szz[1],
                     p.sxy[0], p.sxy[1], p.exx, p.eyy, p.exy, p.vsc[0], p.vsc[1]};
    for (float* z : zero) CK(h, cudaMemset(z, 0, sizeof(float) * n));
    CK(h, cudaMemset(h->passive, 0, sizeof(float) * 5 * n));
    if (!h->reinit) {
        TRY(fill(h, p.vol[0], 1.0f, n, s));
        TRY(fill(h, p.vol[1], 1.0f, n, s));
        TRY(fill(h, p.mass, 1.0f, n, s));
        CK(h, cudaMemset(p.psize, 0, sizeof(float) * n));
    }
    return mpm_write_field(h, MPM_FIELD_LOC, loc, on_device, stream);
}

int mpm_write_field(MpmHandle* h, int field, const void* src, int on_device, void* stream) {
    if (!h) return MPM_ERR_INVALID;
    h->gen++;
    if (h->np < 0) return fail(h, MPM_ERR_STATE, "set particles first");
    if (h->np == 0) return MPM_OK;
    if (!src) return fail(h, MPM_ERR_INVALID, "null source");
    cudaStream_t s = S(stream);
    const int64_t n = h->np;
    PSet& p = h->ps[h->pcur];
    if (field == MPM_FIELD_MATERIAL_ID) {
        std::vector<int32_t> mids((size_t)n);
        if (on_device) CK(h, cudaMemcpy(mids.data(), src, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
        else std::memcpy(mids.data(), src, sizeof(int32_t) * n);
        for (int64_t i = 0; i < n; ++i)
            if (mids[i] < 0 || mids[i] >= h->nmat) return fail(h, MPM_ERR_INVALID, "material id out of range");
        const void* d = nullptr;
        TRY(to_device(h, mids.data(), sizeof(int32_t) * n, 0, s, &d));
        CK(h, launch_gather_in_u8(p.mat, p.pid, (int)n, static_cast<const int32_t*>(d), s));
        return sync(h, s);
    }
    if (field == MPM_FIELD_YOUNGS_MODULUS && !h->has_E) {
        TRY(dalloc(h, &h->ps[0].E, n));
        TRY(dalloc(h, &h->ps[1].E, n));
        h->has_E = true;
        bind_particles(h);
        TRY(upload_desc(h));
    }
    if (field == MPM_FIELD_VOLUME || field == MPM_FIELD_MASS) {
        if (h->reinit)
            return fail(h, MPM_ERR_INVALID, "volume and mass are recomputed every step under solve_jit semantics");
    }
    std::vector<float*> c = comps(h, field);
    if (c.empty()) return fail(h, MPM_ERR_INVALID, "field %d is not writable", field);
    const int nc = (int)c.size();
    const void* d = nullptr;
    TRY(to_device(h, src, sizeof(float) * nc * n, on_device, s, &d));
    TRY(write_float_field(h, field, static_cast<const float*>(d), s));
    return sync(h, s);
}

}  // extern "C"

namespace mpm {
namespace host {

// Before the step counter changes to `step`: when its parity changes, swap the
// ping-pong pairs so that the current data stays addressed by the new parity
// (graphs, which hold the descriptor by value, are dropped).
int keep_parity_data(MpmHandle* h, int64_t step) {
    if ((step & 1) == (h->step & 1) || h->np <= 0) return MPM_OK;
    for (int k = 0; k < 2; ++k) {
        PSet& p = h->ps[k];
        std::swap(p.sxx[0], p.sxx[1]);
        std::swap(p.syy[0], p.syy[1]);
        std::swap(p.szz[0], p.szz[1]);
        std::swap(p.sxy[0], p.sxy[1]);
        std::swap(p.rho[0], p.rho[1]);
        std::swap(p.vsc[0], p.vsc[1]);
        std::swap(p.vol[0], p.vol[1]);
    }
    bind_particles(h);
    drop_graphs(h);
    return upload_desc(h);
}

// A float particle field (original order) from device memory `d` into the
// current particle set, on stream s without waiting.
int write_float_field(MpmHandle* h, int field, const float* d, cudaStream_t s) {
    std::vector<float*> c = comps(h, field);
    if (c.empty()) return fail(h, MPM_ERR_INVALID, "field %d is not writable", field);
    const int nc = (int)c.size();
    PSet& p = h->ps[h->pcur];
    TRY(set_ptr_table(h, c, s));
    CK(h, launch_gather_in(h->d_ptrs, nc, p.pid, (int)h->np, d, s));
    if (field == MPM_FIELD_STRESS || field == MPM_FIELD_STRAIN)
        TRY(copy_passive(h, field, const_cast<float*>(d), false, s));
    if (field == MPM_FIELD_LOC && h->initialized) h->needs_resort = true;
    return MPM_OK;
}


// Particle field `field` in original order into the device buffer `d`.
int gather_field(MpmHandle* h, int field, void* d, cudaStream_t s) {
    const int64_t n = h->np;
    PSet& p = h->ps[h->pcur];
    const int nc = ncomp_of(h, field);
    const bool derived = field == MPM_FIELD_ELEMENT_ID || field == MPM_FIELD_MOMENTUM ||
                         ((field == MPM_FIELD_VOLUME || field == MPM_FIELD_MASS) && h->reinit);
    if (derived) {
        if (h->reinit && h->initialized && h->needs_resort &&
            (field == MPM_FIELD_VOLUME || field == MPM_FIELD_MASS))
            TRY(resort(h, s));
        int what = field == MPM_FIELD_ELEMENT_ID ? 0 : field == MPM_FIELD_VOLUME ? 1 : field == MPM_FIELD_MASS ? 2 : 3;
        if (!h->initialized && (what == 1 || what == 2))
            return fail(h, MPM_ERR_STATE, "initialize first");
        CK(h, launch_derived_out(h->ds, h->ndim, (int)n, parity(h), h->reinit, what, h->ps[h->pcur].pid, d, s));
    } else if (field == MPM_FIELD_MATERIAL_ID) {
        CK(h, launch_scatter_out_u8(p.mat, p.pid, (int)n, static_cast<int32_t*>(d), s));
    } else {
        std::vector<float*> c = comps(h, field);
        if (c.empty() || (field == MPM_FIELD_YOUNGS_MODULUS && !h->has_E))
            return fail(h, MPM_ERR_INVALID, "field %d is not readable", field);
        TRY(set_ptr_table(h, c, s));
        CK(h, launch_scatter_out(h->d_ptrs, nc, p.pid, (int)n, static_cast<float*>(d), s));
        if (field == MPM_FIELD_STRESS || field == MPM_FIELD_STRAIN)
            TRY(copy_passive(h, field, static_cast<float*>(d), true, s));
    }
    return MPM_OK;
}

}  // namespace host
}  // namespace mpm

extern "C" {

int mpm_read_field(MpmHandle* h, int field, void* dst, int on_device, void* stream) {
    if (!h) return MPM_ERR_INVALID;
    if (h->np < 0) return fail(h, MPM_ERR_STATE, "set particles first");
    if (h->np == 0) return MPM_OK;
    if (!dst) return fail(h, MPM_ERR_INVALID, "null destination");
    if (field < 0 || field >= MPM_FIELD_COUNT) return fail(h, MPM_ERR_INVALID, "unknown field %d", field);
    cudaStream_t s = S(stream);
    const size_t bytes = sizeof(float) * ncomp_of(h, field) * h->np;
    void* d = on_device ? dst : nullptr;
    if (!on_device) {
        TRY(ensure_stage(h, bytes));
        d = h->stage;
    }
    TRY(gather_field(h, field, d, s));
    if (!on_device) CK(h, cudaMemcpyAsync(dst, d, bytes, cudaMemcpyDeviceToHost, s));
    return sync(h, s);
}

int mpm_output_enqueue(MpmHandle* h, int nfields, const int* fields, void* host_dst,
                       size_t host_dst_bytes, void* stream, int64_t* ticket) {
    if (!h) return MPM_ERR_INVALID;
    if (h->np < 0) return fail(h, MPM_ERR_STATE, "set particles first");
    if (nfields < 1 || !fields || !host_dst || !ticket)
        return fail(h, MPM_ERR_INVALID, "need at least one field, a destination and a ticket");
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, host_dst) != cudaSuccess || at.type != cudaMemoryTypeHost) {
        cudaGetLastError();
        return fail(h, MPM_ERR_INVALID, "host_dst must be pinned host memory (mpm_host_alloc)");
    }
    cudaStream_t s = S(stream);
    size_t total = 0;
    for (int k = 0; k < nfields; ++k) {
        if (fields[k] < 0 || fields[k] >= MPM_FIELD_COUNT)
            return fail(h, MPM_ERR_INVALID, "unknown field %d", fields[k]);
        total += sizeof(float) * ncomp_of(h, fields[k]) * h->np;
    }
    if (host_dst_bytes < total)
        return fail(h, MPM_ERR_INVALID, "host_dst holds %zu bytes, the fields need %zu", host_dst_bytes,
                    total);
    if (h->out_stage_bytes < total) {
        CK(h, cudaStreamSynchronize(s));      // copies from the old buffer are done
        dfree(h, h->out_stage);
        h->out_stage = nullptr;
        h->out_stage_bytes = 0;
        TRY(dalloc(h, reinterpret_cast<char**>(&h->out_stage), total));
        h->out_stage_bytes = total;
    }
    const int slot = (int)(h->out_tickets % MpmHandle::OUT_SLOTS);
    if (!h->out_ev[slot]) CK(h, cudaEventCreateWithFlags(&h->out_ev[slot], cudaEventDisableTiming));
    size_t off = 0;
    for (int k = 0; k < nfields; ++k) {
        if (h->np > 0) TRY(gather_field(h, fields[k], static_cast<char*>(h->out_stage) + off, s));
        off += sizeof(float) * ncomp_of(h, fields[k]) * h->np;
    }
    if (total) CK(h, cudaMemcpyAsync(host_dst, h->out_stage, total, cudaMemcpyDeviceToHost, s));
    CK(h, cudaEventRecord(h->out_ev[slot], s));
    *ticket = h->out_tickets++;
    return MPM_OK;
}

int mpm_output_wait(MpmHandle* h, int64_t ticket) {
    if (!h) return MPM_ERR_INVALID;
    if (ticket < 0 || ticket >= h->out_tickets || ticket < h->out_tickets - MpmHandle::OUT_SLOTS)
        return MPM_ERR_INVALID;
    cudaEvent_t e = h->out_ev[ticket % MpmHandle::OUT_SLOTS];
    return cudaEventSynchronize(e) == cudaSuccess ? MPM_OK : MPM_ERR_CUDA;
}

int mpm_host_alloc(size_t bytes, void** p) {
    if (!p) return MPM_ERR_INVALID;
    *p = nullptr;
    if (bytes == 0) return MPM_OK;
    if (cudaHostAlloc(p, bytes, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return MPM_ERR_CUDA;
    }
    return MPM_OK;
}

int mpm_host_free(void* p) {
    if (!p) return MPM_OK;
    return cudaFreeHost(p) == cudaSuccess ? MPM_OK : MPM_ERR_CUDA;
}

int mpm_set_tractions(MpmHandle* h, int n, const int64_t* pid, const int32_t* dir,
                      const double* traction, const int32_t* function, void* stream) {
    if (!h) return MPM_ERR_INVALID;
    h->gen++;
    if (h->np < 0) return fail(h, MPM_ERR_STATE, "set particles first");
    if (h->ndim == 1 && n > 0) return fail(h, MPM_ERR_UNSUPPORTED, "particle tractions are not available in 1-D");
    const int64_t np = h->np;
    cudaStream_t s = S(stream);
    if (n <= 0) {
        h->has_trac = false;
        bind_particles(h);
        return upload_desc(h);
    }
    std::vector<int8_t> fn((size_t)(2 * np), 0);
    std::vector<double> tau((size_t)(2 * np), 0.0);
    for (int i = 0; i < n; ++i) {
        const int64_t q = pid[i];
        const int d = dir[i];
        if (q < 0 || q >= np) return fail(h, MPM_ERR_INVALID, "traction particle id out of range");
        if (d != 0 && d != 1) return fail(h, MPM_ERR_INVALID, "traction dir must be 0 or 1");
        if (function[i] < -1 || function[i] >= h->nfn) return fail(h, MPM_ERR_INVALID, "traction function out of range");
        const int8_t code = (int8_t)(function[i] < 0 ? 1 : function[i] + 2);
        int8_t& f = fn[2 * q + d];
        if (f != 0 && f != code)
            return fail(h, MPM_ERR_UNSUPPORTED, "particle %lld has tractions with different time functions in one direction", (long long)q);
        f = code;
        tau[2 * q + d] += traction[i];
    }
    std::vector<float> tau32(tau.begin(), tau.end());
    if (!h->has_trac) {
        for (int k = 0; k < 2; ++k) {
            if (!h->ps[k].tr_fn) TRY(dalloc(h, &h->ps[k].tr_fn, 2 * np));
            if (!h->ps[k].tr_tau) TRY(dalloc(h, &h->ps[k].tr_tau, 2 * np));
        }
    }
    PSet& p = h->ps[h->pcur];
    TRY(ensure_stage(h, sizeof(float) * 2 * np + 2 * np + 64));
    char* st = static_cast<char*>(h->stage);
    CK(h, cudaMemcpyAsync(st, tau32.data(), sizeof(float) * 2 * np, cudaMemcpyHostToDevice, s));
    char* st8 = st + ((sizeof(float) * 2 * np + 63) / 64) * 64;
    CK(h, cudaMemcpyAsync(st8, fn.data(), 2 * np, cudaMemcpyHostToDevice, s));
    CK(h, launch_gather_pair_u32(reinterpret_cast<const uint32_t*>(st), reinterpret_cast<uint32_t*>(p.tr_tau), p.pid, (int)np, s));
    CK(h, launch_gather_pair_u8(reinterpret_cast<const uint8_t*>(st8), reinterpret_cast<uint8_t*>(p.tr_fn), p.pid, (int)np, s));
    h->has_trac = true;
    bind_particles(h);
    drop_graphs(h);
    CK(h, cudaMemcpyAsync(h->ds, &h->hs, sizeof(SimDev), cudaMemcpyHostToDevice, s));
    return sync(h, s);
}

int mpm_set_particle_velocity_constraints(MpmHandle* h, int n, const int64_t* pid, const int32_t* dir,
                                          const double* velocity, void* stream) {
    if (!h) return MPM_ERR_INVALID;
    h->gen++;
    if (h->np < 0) return fail(h, MPM_ERR_STATE, "set particles first");
    const int64_t np = h->np;
    cudaStream_t s = S(stream);
    TRY(sync(h, s));
    if (n <= 0 || np == 0) {
        h->has_pvc = false;
        bind_particles(h);
        drop_graphs(h);
        return upload_desc(h);
    }
    if (!pid || !dir || !velocity) return fail(h, MPM_ERR_INVALID, "null constraint list");
    std::vector<uint8_t> code((size_t)(2 * np), 0);
    std::vector<float> vel;
    for (int i = 0; i < n; ++i) {
        const int64_t q = pid[i];
        const int d = dir[i];
        if (q < 0 || q >= np) return fail(h, MPM_ERR_INVALID, "constrained particle id out of range");
        if (d < 0 || d >= h->ndim) return fail(h, MPM_ERR_INVALID, "constraint dir out of range");
        const float v = (float)velocity[i];
        int slot = -1;
        for (size_t k = 0; k < vel.size(); ++k)
            if (std::memcmp(&vel[k], &v, sizeof v) == 0) slot = (int)k;
        if (slot < 0) {
            if (vel.size() >= 255) return fail(h, MPM_ERR_UNSUPPORTED, "more than 255 distinct particle velocities");
            vel.push_back(v);
            slot = (int)vel.size() - 1;
        }
        code[2 * q + d] = (uint8_t)(slot + 1);   // later entries win, as for nodes
    }
    for (int k = 0; k < 2; ++k)
        if (!h->ps[k].pvc) TRY(dalloc(h, &h->ps[k].pvc, 2 * np));
    if (!h->d_pvc_vel) TRY(dalloc(h, &h->d_pvc_vel, 256));
    CK(h, cudaMemcpy(h->d_pvc_vel, vel.data(), sizeof(float) * vel.size(), cudaMemcpyHostToDevice));
    PSet& p = h->ps[h->pcur];
    TRY(ensure_stage(h, 2 * np));
    CK(h, cudaMemcpyAsync(h->stage, code.data(), 2 * np, cudaMemcpyHostToDevice, s));
    CK(h, launch_gather_pair_u8(static_cast<const uint8_t*>(h->stage), p.pvc, p.pid, (int)np, s));
    h->has_pvc = true;
    bind_particles(h);
    drop_graphs(h);
    CK(h, cudaMemcpyAsync(h->ds, &h->hs, sizeof(SimDev), cudaMemcpyHostToDevice, s));
    return sync(h, s);
}

int mpm_read_nodal_field(MpmHandle* h, int field, float* dst, int on_device, void* stream) {
    if (!h || !dst) return MPM_ERR_INVALID;
    cudaStream_t s = S(stream);
    const bool line = h->ndim == 1;
    const int nc = field == MPM_NODE_MASS || line ? 1 : 2;
    const size_t bytes = sizeof(float) * nc * h->nn;
    float* d = dst;
    if (!on_device) {
        TRY(ensure_stage(h, bytes));
        d = static_cast<float*>(h->stage);
    }
    if (field == MPM_NODE_MASS) CK(h, cudaMemcpyAsync(d, h->nm, bytes, cudaMemcpyDeviceToDevice, s));
    else if (field == MPM_NODE_VELOCITY && line) CK(h, cudaMemcpyAsync(d, h->nvbx, bytes, cudaMemcpyDeviceToDevice, s));
    else if (field == MPM_NODE_ACCELERATION && line) CK(h, cudaMemcpyAsync(d, h->nax, bytes, cudaMemcpyDeviceToDevice, s));
    else if (field == MPM_NODE_VELOCITY) CK(h, launch_interleave2(h->nvbx, h->nvby, h->nn, d, s));
    else if (field == MPM_NODE_ACCELERATION) CK(h, launch_interleave2(h->nax, h->nay, h->nn, d, s));
    else if (field == MPM_NODE_MOMENTUM)
        CK(h, launch_node_momentum(h->nm, h->nvbx, line ? nullptr : h->nvby, h->nn, d, s));
    else return fail(h, MPM_ERR_INVALID, "unknown nodal field %d", field);
    if (!on_device) CK(h, cudaMemcpyAsync(dst, d, bytes, cudaMemcpyDeviceToHost, s));
    return sync(h, s);
}

int mpm_write_nodal_field(MpmHandle* h, int field, const float* src, int on_device, void* stream) {
    if (!h || !src) return MPM_ERR_INVALID;
    h->gen++;
    cudaStream_t s = S(stream);
    const bool line = h->ndim == 1;
    const int nc = field == MPM_NODE_MASS || line ? 1 : 2;
    const void* d = nullptr;
    TRY(to_device(h, src, sizeof(float) * nc * h->nn, on_device, s, &d));
    const float* df = static_cast<const float*>(d);
    if (field == MPM_NODE_MASS) CK(h, cudaMemcpyAsync(h->nm, df, sizeof(float) * h->nn, cudaMemcpyDeviceToDevice, s));
    else if (field == MPM_NODE_VELOCITY && line)
        CK(h, cudaMemcpyAsync(h->nvbx, df, sizeof(float) * h->nn, cudaMemcpyDeviceToDevice, s));
    else if (field == MPM_NODE_ACCELERATION && line)
        CK(h, cudaMemcpyAsync(h->nax, df, sizeof(float) * h->nn, cudaMemcpyDeviceToDevice, s));
    else if (field == MPM_NODE_VELOCITY) CK(h, launch_deinterleave2(df, h->nn, h->nvbx, h->nvby, s));
    else if (field == MPM_NODE_ACCELERATION) CK(h, launch_deinterleave2(df, h->nn, h->nax, h->nay, s));
    else return fail(h, MPM_ERR_INVALID, "nodal field %d is not writable", field);
    return sync(h, s);
}

int mpm_initialize(MpmHandle* h, void* stream) {
    if (!h) return MPM_ERR_INVALID;
    h->gen++;
    if (h->np < 0) return fail(h, MPM_ERR_STATE, "set particles first");
    cudaStream_t s = S(stream);
    TRY(clear_status(h, s));
    TRY(resort(h, s));
    if (!h->reinit && h->np > 0) {
        if (h->ndim == 1) TRY(line_setup_volume(h, s));
        else CK(h, launch_setup_volume(h->ds, (int)h->np, parity(h), s));
    }
    TRY(read_ctl(h, s));
    int st = 0;
    TRY(check_status(h, st));
    h->initialized = true;
    return MPM_OK;
}

int mpm_run_phase(MpmHandle* h, int phase, void* stream) {
    if (!h) return MPM_ERR_INVALID;
    h->gen++;
    if (!h->initialized) return fail(h, MPM_ERR_STATE, "initialize first");
    if (phase < 0 || phase > 2) return fail(h, MPM_ERR_INVALID, "phase must be 0, 1 or 2");
    if (h->ndim == 1) return fail(h, MPM_ERR_UNSUPPORTED, "single phases are not available in 1-D");
    cudaStream_t s = S(stream);
    if (phase == 0 && h->needs_resort) TRY(resort(h, s));
    if (phase == 0) TRY(classify_tiles(h, s));
    TRY(launch_phase(h, phase, 0, s));
    if (phase == 2) {
        CK(h, launch_advance_step(h->ctl, 1, s));
        h->step++;
        TRY(read_ctl(h, s));
        int st = 0;
        TRY(check_status(h, st));
        if (st & (ST_DRIFTED | ST_DRIFT_VIOLATION)) h->needs_resort = true;
        if (st & ST_DRIFT_VIOLATION)
            return fail(h, MPM_ERR_CFL, "a particle moved two cells from its sort-cell within one phase sequence");
        TRY(clear_status(h, s));
    }
    return sync(h, s);
}

int mpm_step(MpmHandle* h, int nsteps, void* stream) {
    if (!h) return MPM_ERR_INVALID;
    h->gen++;
    if (!h->initialized) return fail(h, MPM_ERR_STATE, "initialize first");
    if (nsteps < 0) return fail(h, MPM_ERR_INVALID, "nsteps must be >= 0");
    if (h->np <= 0) {
        h->step += nsteps;
        Control c{};
        c.step = (int)h->step;
        *h->h_ctl = c;
        CK(h, cudaMemcpy(h->ctl, h->h_ctl, sizeof c, cudaMemcpyHostToDevice));
        return MPM_OK;
    }
    cudaStream_t s = S(stream);
    if (h->ndim == 1) {   // Linear1D: re-sorted every step, status checked at the end
        for (int t = 0; t < nsteps; ++t) TRY(line_step(h, s));
        TRY(read_ctl(h, s));
        int st = h->h_ctl->status;
        TRY(check_status(h, st));
        TRY(clear_status(h, s));
        return sync(h, s);
    }
    while (nsteps > 0) {
        const int B = nsteps < h->block_steps ? nsteps : h->block_steps;
        if (h->needs_resort) TRY(resort(h, s));
        const int64_t step0 = h->step;
        TRY(take_snapshot(h, s));
        TRY(run_graph(h, B, s));
        h->step += B;
        TRY(read_ctl(h, s));
        // a two-cell drift corrupts the rest of the block (a particle may even be
        // thrown out of the mesh by it): roll back before judging anything else
        int st = h->h_ctl->status;
        if (st & ST_DRIFT_VIOLATION) TRY(replay_block(h, step0, B, st, s));
        else TRY(check_status(h, st));
        h->needs_resort = (st & ST_DRIFTED) != 0;
        TRY(clear_status(h, s));
        nsteps -= B;
    }
    return sync(h, s);
}

int mpm_get_step(const MpmHandle* h, int64_t* step) {
    if (!h || !step) return MPM_ERR_INVALID;
    *step = h->step;
    return MPM_OK;
}

int mpm_set_step(MpmHandle* h, int64_t step) {
    if (!h || step < 0 || step > 0x7fffffff) return MPM_ERR_INVALID;
    h->gen++;
    TRY(keep_parity_data(h, step));
    h->step = step;
    h->h_ctl->step = (int)step;
    CK(h, cudaMemcpy(&h->ctl->step, &h->h_ctl->step, sizeof(int), cudaMemcpyHostToDevice));
    return MPM_OK;
}

int mpm_time_phases(MpmHandle* h, int nsteps, float* ms_out, void* stream) {
    if (!h || !ms_out || nsteps < 1) return MPM_ERR_INVALID;
    h->gen++;
    if (!h->initialized) return fail(h, MPM_ERR_STATE, "initialize first");
    if (h->ndim == 1) return fail(h, MPM_ERR_UNSUPPORTED, "phase timing is not available in 1-D");
    cudaStream_t s = S(stream);
    if (h->needs_resort) TRY(resort(h, s));
    TRY(classify_tiles(h, s));
    std::vector<cudaEvent_t> ev((size_t)3 * nsteps + 1);
    for (auto& e : ev) CK(h, cudaEventCreate(&e));
    int r = MPM_OK;
    CK(h, cudaEventRecord(ev[0], s));
    for (int i = 0; i < nsteps && r == MPM_OK; ++i)
        for (int p = 0; p < 3 && r == MPM_OK; ++p) {
            r = launch_phase(h, p, 0, s);
            if (r == MPM_OK && p == 2) CK(h, launch_advance_step(h->ctl, 1, s));
            if (r == MPM_OK) CK(h, cudaEventRecord(ev[3 * i + p + 1], s));
        }
    CK(h, cudaStreamSynchronize(s));
    for (int p = 0; p < 3; ++p) ms_out[p] = 0.0f;
    if (r == MPM_OK)
        for (int i = 0; i < nsteps; ++i)
            for (int p = 0; p < 3; ++p) {
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, ev[3 * i + p], ev[3 * i + p + 1]);
                ms_out[p] += ms;
            }
    for (auto& e : ev) cudaEventDestroy(e);
    TRY(r);
    h->step += nsteps;
    TRY(read_ctl(h, s));
    int st = 0;
    TRY(check_status(h, st));
    h->needs_resort = (st & (ST_DRIFTED | ST_DRIFT_VIOLATION)) != 0;
    TRY(clear_status(h, s));
    return MPM_OK;
}

int mpm_set_gravity(MpmHandle* h, double gx, double gy) {
    if (!h) return MPM_ERR_INVALID;
    h->gen++;
    h->gx = (float)gx;
    h->gy = (float)gy;
    h->hs.gx = h->gx;
    h->hs.gy = h->gy;
    return upload_desc(h);
}

int mpm_set_block_steps(MpmHandle* h, int steps) {
    if (!h || steps < 1) return MPM_ERR_INVALID;
    h->block_steps = steps;
    return MPM_OK;
}

int mpm_device_name(int device, char* name, int len) {
    if (!name || len < 1) return MPM_ERR_INVALID;
    cudaDeviceProp prop{};
    const cudaError_t e = cudaGetDeviceProperties(&prop, device);
    if (e != cudaSuccess) {
        cudaGetLastError();
        name[0] = 0;
        return MPM_ERR_CUDA;
    }
    snprintf(name, (size_t)len, "%s (sm_%d%d, %d SMs)", prop.name, prop.major, prop.minor,
             prop.multiProcessorCount);
    return MPM_OK;
}

int mpm_set_empty_split(MpmHandle* h, int min_empty) {
    if (!h) return MPM_ERR_INVALID;
    if (min_empty < 0) return fail(h, MPM_ERR_INVALID, "min_empty is negative");
    h->empty_split_min = min_empty;   // applies from the next classification
    return MPM_OK;
}

int mpm_set_kernel_variant(MpmHandle* h, int nk_ctas, int g2p_ctas, int forces_lpc) {
    if (!h) return MPM_ERR_INVALID;
    if ((nk_ctas != 2 && nk_ctas != 3) || (g2p_ctas != 2 && g2p_ctas != 3))
        return fail(h, MPM_ERR_INVALID, "kernel builds exist for 2 or 3 CTAs per SM");
    if (forces_lpc < 0 || forces_lpc > 2) return fail(h, MPM_ERR_INVALID, "forces_lpc is 0, 1 or 2");
    if (nk_ctas != h->nk_ctas || g2p_ctas != h->g2p_ctas || forces_lpc != h->forces_lpc) {
        h->nk_ctas = nk_ctas;
        h->g2p_ctas = g2p_ctas;
        h->forces_lpc = forces_lpc;
        drop_graphs(h);   // the captured graphs hold the other builds
    }
    return MPM_OK;
}

int mpm_get_counters(const MpmHandle* h, int64_t* resorts, int64_t* rollbacks) {
    if (!h) return MPM_ERR_INVALID;
    if (resorts) *resorts = h->resorts;
    if (rollbacks) *rollbacks = h->rollbacks;
    return MPM_OK;
}

}  // extern "C"
