// Differentiation of the explicit step: a checkpointed forward run
// (mpm_record) and the hand-written discrete adjoint (mpm_adjoint).
//
// mpm_record advances like mpm_step and keeps a full copy of the simulation
// state at the start of every segment of K steps (and at the end), plus the
// steps before which the particles were re-sorted.  mpm_adjoint walks the
// segments backwards: it restores the segment's checkpoint, re-runs its K
// steps while copying each step's start state and nodal results into a tape
// (re-sorting at the recorded steps, so the storage order of every step
// matches the recorded run), then runs the four reverse passes of
// mpm_adjoint.h for each step from the last to the first.  A segment without
// a re-sort re-runs and reverses as two cached CUDA graphs; one with a
// re-sort goes step by step.  The adjoint arrays
// follow the storage order of the step being reversed; where a re-sort
// separates two steps they are permuted through the original particle order,
// and after a segment they are left in the order of its checkpoint, which is
// the order the re-run of the previous segment ends in (the re-run is checked
// to reproduce the recorded state bit for bit).
// Memory: one checkpoint per segment (the particle state, cell starts and
// persistent nodal velocity) and a tape of K steps (9 floats per particle, 7
// per node and 1 byte per cell per step; one more float per particle for the
// volume under solve semantics and one for the volumetric strain of a run
// with Newtonian particles).
//
// mpm_batch_record / mpm_batch_adjoint do the same for every simulation of a
// batch in lockstep: each re-run step, tape copy and reverse pass is one
// launch for all simulations (segmented copies with a slot offset, and the
// reverse passes over a table of per-simulation arguments).
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <vector>

#include "mpm_adjoint.h"
#include "mpm_batch.h"
#include "mpm_handle.h"

using namespace mpm;
using namespace mpm::host;


namespace mpm {

namespace {

constexpr int NLAM = 12;   // adjoint arrays: x y vx vy sxx syy szz sxy rho E vol vsc
constexpr int NTP = 9;     // tape per particle: x y vx vy sxx syy szz sxy rho
constexpr int NTN = 7;     // tape per node: m vAx vAy vBx vBy aBx aBy
constexpr int NPS = 5;     // per-particle scratch: r0b r1b r3b c0b c1b
constexpr int NNS = 8;     // per-node scratch: fbx fby mb vabx vaby qbx qby mbt

struct Epoch {               // arrays of one sort epoch inside a segment
    int* pid = nullptr;
    uint8_t* mat = nullptr;
    float* E = nullptr;
    int* cstart = nullptr;
    int8_t* tr_fn = nullptr;   // particle tractions (2 per particle), when present
    float* tr_tau = nullptr;
    uint8_t* pvc = nullptr;    // velocity constraint codes (2 per particle), when present
    float* mass = nullptr;     // solve semantics: the constant mass and size
    float* psize = nullptr;
};

}  // namespace

struct AdjointState {
    int K = 0, nseg = 0;
    int64_t step0 = 0, nsteps = 0;
    uint64_t gen = 0;
    bool valid = false, recording = false;
    std::vector<int64_t> resort_steps;
    std::vector<Checkpoint> ck;   // ck[s]: start of segment s; ck[nseg]: end state
    // sized for np_alloc particles and tape_slots steps
    int64_t np_alloc = -1;
    int tape_slots = 0;
    float* tp[NTP] = {};
    float* tvol = nullptr;     // volume at each step start (solve semantics only)
    float* tvsc = nullptr;     // centroid volumetric strain at each step start (Newtonian only)
    uint8_t* tflag = nullptr;
    float* tn[NTN] = {};
    std::vector<Epoch> epochs;
    std::vector<int> epoch_of;
    int nep = 0;               // epochs captured in the current segment
    int64_t seg_first = 0;     // first step of the segment being reversed
    float* lam[NLAM] = {};
    float* lam_tmp = nullptr;
    float** d_lam = nullptr;
    float* pscr[NPS] = {};
    float* nscr[NNS] = {};
    int* cnt = nullptr;
    int* mismatch = nullptr;   // device counter of the re-run check
    int* h_mismatch = nullptr; // pinned
    // CUDA graphs of whole segments without a re-sort: the re-run with its
    // tape copies (keyed by 2 * length + start parity) and the reverse steps
    // (keyed by length).  They hold the step descriptor and every buffer
    // pointer by value, so they are dropped when the handle's step graphs are
    // (g_gen != graph_gen) and whenever a buffer here is (re)allocated.
    std::map<int64_t, cudaGraphExec_t> g_rerun, g_rev;
    SegBuf g_tp[2], g_tn;      // tape copy tables of the re-run graphs
    uint64_t g_gen = ~0ull;
};

// Scratch of a batched adjoint (owned by the batch).
struct BatchAdjoint {
    AdjStep* d_bases = nullptr;
    AdjStep* d_table = nullptr;
    std::vector<AdjStep> bases;
    int2* part_blocks = nullptr;
    int n_part_blocks = 0;
    SegBuf tape_p[2], tape_n, misc;
    int* mismatch = nullptr;
    int* h_mismatch = nullptr;
    // graphs of one-epoch segments: the re-run (keyed by length and tile
    // counts) and the reverse steps (length, tiles, particle blocks); valid
    // for the buffers and kernel builds in `gsig`
    std::map<int64_t, cudaGraphExec_t> g_rerun, g_rev;
    std::vector<uintptr_t> gsig;
};

namespace {

void drop_adj_graphs(AdjointState* a) {
    for (auto& kv : a->g_rerun) cudaGraphExecDestroy(kv.second);
    for (auto& kv : a->g_rev) cudaGraphExecDestroy(kv.second);
    a->g_rerun.clear();
    a->g_rev.clear();
    for (SegBuf& b : a->g_tp) segbuf_free(b);
    segbuf_free(a->g_tn);
    a->g_gen = ~0ull;
}

void free_buffers(MpmHandle* h, AdjointState* a) {
    drop_adj_graphs(a);
    for (auto& c : a->ck) checkpoint_free(h, c);
    a->ck.clear();
    for (float*& p : a->tp) { dfree(h, p); p = nullptr; }
    for (float*& p : a->tn) { dfree(h, p); p = nullptr; }
    dfree(h, a->tvol);
    a->tvol = nullptr;
    dfree(h, a->tvsc);
    a->tvsc = nullptr;
    dfree(h, a->tflag);
    a->tflag = nullptr;
    a->tape_slots = 0;
    for (Epoch& e : a->epochs) {
        dfree(h, e.pid);
        dfree(h, e.mat);
        dfree(h, e.E);
        dfree(h, e.cstart);
        dfree(h, e.tr_fn);
        dfree(h, e.tr_tau);
        dfree(h, e.pvc);
        dfree(h, e.mass);
        dfree(h, e.psize);
    }
    a->epochs.clear();
    for (float*& p : a->lam) { dfree(h, p); p = nullptr; }
    for (float*& p : a->pscr) { dfree(h, p); p = nullptr; }
    for (float*& p : a->nscr) { dfree(h, p); p = nullptr; }
    dfree(h, a->lam_tmp);
    dfree(h, a->d_lam);
    dfree(h, a->cnt);
    dfree(h, a->mismatch);
    if (a->h_mismatch) cudaFreeHost(a->h_mismatch);
    a->mismatch = nullptr;
    a->h_mismatch = nullptr;
    a->lam_tmp = nullptr;
    a->d_lam = nullptr;
    a->cnt = nullptr;
    a->np_alloc = -1;
    a->valid = false;
}

// Drop everything sized for another particle count.
void fit(MpmHandle* h, AdjointState* a) {
    if (a->np_alloc != h->np) {
        free_buffers(h, a);
        a->np_alloc = h->np;
    }
}

int save_checkpoint(MpmHandle* h, AdjointState* a, size_t idx, std::vector<CopySeg>& v) {
    if (a->ck.size() <= idx) a->ck.resize(idx + 1);
    TRY(checkpoint_alloc(h, a->ck[idx]));
    checkpoint_segments(h, a->ck[idx], true, v);
    return MPM_OK;
}

int restore_checkpoint(MpmHandle* h, Checkpoint& c, cudaStream_t s) {
    std::vector<CopySeg> v;
    checkpoint_segments(h, c, false, v);
    TRY(run_segments(h, h->segbuf, v, s));
    TRY(clear_status(h, s));
    return sync(h, s);
}

// Particle slots between consecutive tape slots (np rounded up to 4).
size_t tape_stride(const MpmHandle* h) { return ((size_t)h->np + 3) & ~(size_t)3; }

int ensure_adjoint_buffers(MpmHandle* h, AdjointState* a, int slots, cudaStream_t s) {
    // particle arrays and tape slots hold a multiple of 4 slots, so that every
    // slot starts on a 16-byte boundary for the reverse node passes' 16-byte
    // row staging (which may read up to 3 slots past a row's end)
    const size_t np = ((size_t)h->np + 3) & ~(size_t)3, nn = (size_t)h->nn;
    bool newtonian = false;
    for (const MatDev& m : h->mats) newtonian = newtonian || m.type == MAT_NEWTONIAN;
    if (a->tape_slots < slots || (!h->reinit && !a->tvol) || (newtonian && !a->tvsc)) {
        drop_adj_graphs(a);
        for (float*& p : a->tp) { dfree(h, p); p = nullptr; }
        dfree(h, a->tvol);
        a->tvol = nullptr;
        dfree(h, a->tvsc);
        a->tvsc = nullptr;
        for (float*& p : a->tn) { dfree(h, p); p = nullptr; }
        dfree(h, a->tflag);
        a->tflag = nullptr;
        a->tape_slots = 0;
        for (float*& p : a->tp) TRY(dalloc(h, &p, np * slots));
        if (!h->reinit) TRY(dalloc(h, &a->tvol, np * slots));
        if (newtonian) TRY(dalloc(h, &a->tvsc, np * slots));
        for (float*& p : a->tn) TRY(dalloc(h, &p, nn * slots));
        TRY(dalloc(h, &a->tflag, (size_t)h->ncell * slots));
        a->tape_slots = slots;
    }
    if (!a->lam[0]) {
        drop_adj_graphs(a);
        for (float*& p : a->lam) TRY(dalloc(h, &p, np));
        for (float*& p : a->pscr) TRY(dalloc(h, &p, np));
        for (float*& p : a->nscr) TRY(dalloc(h, &p, nn));
        TRY(dalloc(h, &a->lam_tmp, np * NLAM));
        TRY(dalloc(h, &a->d_lam, NLAM));
        TRY(dalloc(h, &a->cnt, (size_t)h->ncell));
        TRY(dalloc(h, &a->mismatch, 1));
        CK(h, cudaMallocHost(&a->h_mismatch, sizeof(int)));
        CK(h, cudaMemcpyAsync(a->d_lam, a->lam, sizeof(float*) * NLAM, cudaMemcpyHostToDevice, s));
        TRY(sync(h, s));
    }
    return MPM_OK;
}

void add_seg(std::vector<CopySeg>& v, const void* src, void* dst, size_t bytes, size_t step) {
    CopySeg c;
    c.src = src;
    c.dst = dst;
    c.bytes = bytes;
    c.dst_step = step;
    v.push_back(c);
}

// Segments copying the current sort epoch's order-dependent arrays into epoch slot e.
int epoch_segments(MpmHandle* h, AdjointState* a, size_t e, std::vector<CopySeg>& v) {
    const size_t np = (size_t)h->np;
    if (a->epochs.size() <= e) {
        drop_adj_graphs(a);
        Epoch ep;
        TRY(dalloc(h, &ep.pid, np));
        TRY(dalloc(h, &ep.mat, np));
        TRY(dalloc(h, &ep.cstart, (size_t)h->ncell + 2));
        a->epochs.push_back(ep);
    }
    Epoch& ep = a->epochs[e];
    if (h->has_E && !ep.E) {
        drop_adj_graphs(a);
        TRY(dalloc(h, &ep.E, np));
    }
    if (h->has_trac && !ep.tr_fn) {
        drop_adj_graphs(a);
        TRY(dalloc(h, &ep.tr_fn, 2 * np));
        TRY(dalloc(h, &ep.tr_tau, 2 * np));
    }
    if (h->has_pvc && !ep.pvc) {
        drop_adj_graphs(a);
        TRY(dalloc(h, &ep.pvc, 2 * np));
    }
    if (!h->reinit && !ep.mass) {
        drop_adj_graphs(a);
        TRY(dalloc(h, &ep.mass, np));
        TRY(dalloc(h, &ep.psize, np));
    }
    const PSet& p = h->ps[h->pcur];
    add_seg(v, p.pid, ep.pid, sizeof(int) * np, 0);
    add_seg(v, p.mat, ep.mat, np, 0);
    if (h->has_E) add_seg(v, p.E, ep.E, sizeof(float) * np, 0);
    if (h->has_trac) {
        add_seg(v, p.tr_fn, ep.tr_fn, 2 * np, 0);
        add_seg(v, p.tr_tau, ep.tr_tau, sizeof(float) * 2 * np, 0);
    }
    if (h->has_pvc) add_seg(v, p.pvc, ep.pvc, 2 * np, 0);
    if (!h->reinit) {
        add_seg(v, p.mass, ep.mass, sizeof(float) * np, 0);
        add_seg(v, p.psize, ep.psize, sizeof(float) * np, 0);
    }
    add_seg(v, h->cstart[h->cs_cur], ep.cstart, sizeof(int) * ((size_t)h->ncell + 2), 0);
    return MPM_OK;
}

int capture_epoch(MpmHandle* h, AdjointState* a, cudaStream_t s) {
    std::vector<CopySeg> v;
    TRY(epoch_segments(h, a, (size_t)a->nep, v));
    a->nep++;
    return run_segments(h, h->segbuf, v, s);
}

// Tape copies of a step that starts with ping-pong parity `par`: the particle
// state and drift flags (before the step) into slot 0 + t * stride.
void tape_particle_segments(MpmHandle* h, AdjointState* a, int par, std::vector<CopySeg>& v) {
    const PSet& p = h->ps[h->pcur];
    const size_t np = (size_t)h->np, stride = tape_stride(h);
    const float* src[NTP] = {p.x, p.y, p.vx, p.vy, p.sxx[par], p.syy[par], p.szz[par],
                             p.sxy[par], p.rho[par]};
    for (int k = 0; k < NTP; ++k) add_seg(v, src[k], a->tp[k], sizeof(float) * np, sizeof(float) * stride);
    if (!h->reinit) add_seg(v, p.vol[par], a->tvol, sizeof(float) * np, sizeof(float) * stride);
    if (a->tvsc) add_seg(v, p.vsc[par], a->tvsc, sizeof(float) * np, sizeof(float) * stride);
    add_seg(v, h->cflag, a->tflag, (size_t)h->ncell, (size_t)h->ncell);
}

// ... and the nodal results (after the step).
void tape_node_segments(MpmHandle* h, AdjointState* a, std::vector<CopySeg>& v) {
    const size_t nn = (size_t)h->nn;
    const float* src[NTN] = {h->nm, h->nvax, h->nvay, h->nvbx, h->nvby, h->nax, h->nay};
    for (int k = 0; k < NTN; ++k) add_seg(v, src[k], a->tn[k], sizeof(float) * nn, sizeof(float) * nn);
}

// Pairs (re-run state, recorded state of the next checkpoint) for the bitwise check.
void check_segments(MpmHandle* h, AdjointState* a, int seg, std::vector<CopySeg>& v) {
    const Checkpoint& next = a->ck[seg + 1];
    std::vector<float**> f = movable_f32(h, h->ps[h->pcur], false);
    for (size_t i = 0; i < f.size(); ++i) add_seg(v, *f[i], next.f[i], sizeof(float) * h->np, 0);
}

bool resorts_at(const AdjointState* a, int64_t step) {
    return std::binary_search(a->resort_steps.begin(), a->resort_steps.end(), step);
}

// Tape copy tables of the segment graphs, for the handle's current
// descriptors (the previous graphs are dropped when those changed).
int prepare_adj_graphs(MpmHandle* h, AdjointState* a, cudaStream_t s) {
    if (a->g_gen == h->graph_gen) return MPM_OK;
    drop_adj_graphs(a);
    for (int par = 0; par < 2; ++par) {
        std::vector<CopySeg> v;
        tape_particle_segments(h, a, par, v);
        TRY(upload_segments(h, a->g_tp[par], v, s));
    }
    std::vector<CopySeg> vn;
    tape_node_segments(h, a, vn);
    TRY(upload_segments(h, a->g_tn, vn, s));
    a->g_gen = h->graph_gen;
    return MPM_OK;
}

// Capture the launches that `body` issues on the handle's capture stream
// into an executable graph stored at map[key] (if absent), then launch it.
template <class F>
int run_cached_graph(MpmHandle* h, std::map<int64_t, cudaGraphExec_t>& map, int64_t key, cudaStream_t s,
                     F&& body) {
    auto it = map.find(key);
    if (it == map.end()) {
        cudaGraph_t g = nullptr;
        CK(h, cudaStreamBeginCapture(h->cap, cudaStreamCaptureModeThreadLocal));
        const int r = body(h->cap);
        const cudaError_t e = cudaStreamEndCapture(h->cap, &g);
        if (r != MPM_OK || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            if (r != MPM_OK) return r;
            CK(h, e);
        }
        cudaGraphExec_t ex = nullptr;
        const cudaError_t ei = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        CK(h, ei);
        it = map.emplace(key, ex).first;
    }
    CK(h, cudaGraphLaunch(it->second, s));
    return MPM_OK;
}

// Re-run of a segment of `len` steps without a re-sort as one graph: per
// step the tape copy of the start state, the step's kernels (at step offset
// t) and the tape copy of the nodal results; the step counter advances once.
int rerun_graph(MpmHandle* h, AdjointState* a, int len, cudaStream_t s) {
    TRY(prepare_adj_graphs(h, a, s));
    TRY(classify_tiles(h, s));   // the restored checkpoint's sort
    const int par0 = parity(h);
    TRY(run_cached_graph(h, a->g_rerun, seq_key(h, 2 * len + par0), s, [&](cudaStream_t c) -> int {
        for (int t = 0; t < len; ++t) {
            const SegBuf& tp = a->g_tp[(par0 + t) & 1];
            CK(h, launch_copy_segments(tp.blk, tp.nblocks, t, c));
            for (int p = 0; p < 3; ++p) TRY(launch_phase(h, p, t, c));
            CK(h, launch_copy_segments(a->g_tn.blk, a->g_tn.nblocks, t, c));
        }
        CK(h, launch_advance_step(h->ctl, len, c));
        return MPM_OK;
    }));
    h->step += len;
    return MPM_OK;
}

// Re-run segment `seg` of one simulation from its checkpoint, filling tape
// slots 0..len-1, and check that it ends in the next checkpoint's state.
int recompute_segment(MpmHandle* h, AdjointState* a, int seg, int len, cudaStream_t s) {
    TRY(restore_checkpoint(h, a->ck[seg], s));
    const int64_t first = a->ck[seg].step;
    a->seg_first = first;
    a->epoch_of.assign(len, 0);
    a->nep = 0;
    TRY(capture_epoch(h, a, s));
    bool resorts = false;
    for (int t = 0; t < len; ++t) resorts = resorts || resorts_at(a, first + t);
    SegBuf& tp = h->segbuf;
    int tp_par = -1;
    SegBuf tn;
    std::vector<CopySeg> vn;
    tape_node_segments(h, a, vn);
    if (resorts) TRY(upload_segments(h, tn, vn, s));
    int r = resorts ? MPM_OK : rerun_graph(h, a, len, s);
    for (int t = 0; t < len && r == MPM_OK && resorts; ++t) {
        if (resorts_at(a, first + t)) {
            r = resort(h, s);
            if (r == MPM_OK) r = capture_epoch(h, a, s);
            tp_par = -1;
            if (r != MPM_OK) break;
        }
        const int par = parity(h);
        if (par != tp_par) {
            std::vector<CopySeg> v;
            tape_particle_segments(h, a, par, v);
            r = upload_segments(h, tp, v, s);
            if (r != MPM_OK) break;
            tp_par = par;
        }
        if (t == 0 || resorts_at(a, first + t)) {   // the sort of the step (restored or re-sorted)
            r = classify_tiles(h, s);
            if (r != MPM_OK) break;
        }
        cudaError_t e = launch_copy_segments(tp.blk, tp.nblocks, t, s);
        if (e == cudaSuccess) {
            r = launch_steps(h, 1, s);
            h->step++;
        }
        if (e == cudaSuccess && r == MPM_OK)
            e = launch_copy_segments(tn.blk, tn.nblocks, t, s);
        if (e != cudaSuccess) r = fail(h, MPM_ERR_CUDA, "tape copy: %s", cudaGetErrorString(e));
        a->epoch_of[t] = a->nep - 1;
    }
    if (r == MPM_OK) r = read_ctl(h, s);
    segbuf_free(tn);
    TRY(r);
    int st = 0;
    TRY(check_status(h, st));
    // the re-run must end bit for bit in the recorded state of the next checkpoint
    std::vector<CopySeg> vc;
    check_segments(h, a, seg, vc);
    SegBuf cb;
    r = upload_segments(h, cb, vc, s);
    if (r == MPM_OK) {
        cudaError_t e = cudaMemsetAsync(a->mismatch, 0, sizeof(int), s);
        if (e == cudaSuccess) e = launch_compare_segments(cb.blk, cb.nblocks, a->mismatch, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(a->h_mismatch, a->mismatch, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) r = fail(h, MPM_ERR_CUDA, "re-run check: %s", cudaGetErrorString(e));
        if (r == MPM_OK) r = sync(h, s);
    }
    segbuf_free(cb);
    TRY(r);
    if ((st & ST_DRIFT_VIOLATION) || *a->h_mismatch != 0 || h->step != a->ck[seg + 1].step)
        return fail(h, MPM_ERR_STATE,
                    "re-run of steps %lld..%lld did not reproduce the recorded run (%d words differ)",
                    (long long)first, (long long)(first + len - 1), *a->h_mismatch);
    return clear_status(h, s);
}

// Move the adjoint arrays from the storage order `from` to the storage order `to`.
int permute(MpmHandle* h, AdjointState* a, const int* from, const int* to, cudaStream_t s) {
    if (from == to) return MPM_OK;
    const int np = (int)h->np;
    CK(h, launch_scatter_out(a->d_lam, NLAM, from, np, a->lam_tmp, s));
    CK(h, launch_gather_in(a->d_lam, NLAM, to, np, a->lam_tmp, s));
    return MPM_OK;
}

// Reverse-pass arguments with the tape at slot 0 and the epoch of slot t.
AdjStep base_args(MpmHandle* h, AdjointState* a, int epoch) {
    const Epoch& ep = a->epochs[epoch];
    AdjStep A{};
    A.nx = h->nx;
    A.ny = h->ny;
    A.np = (int)h->np;
    A.hx = h->hx;
    A.hy = h->hy;
    A.dt = h->dt;
    A.vol_el = h->vol_el;
    A.gx = h->gx;
    A.gy = h->gy;
    A.velocity_update = h->velocity_update;
    A.ncons = h->d_ncons;
    A.mats = h->d_mats;
    A.cstart = ep.cstart;
    A.mat = ep.mat;
    A.E = h->has_E ? ep.E : nullptr;
    A.tr_fn = h->has_trac ? ep.tr_fn : nullptr;
    A.tr_tau = h->has_trac ? ep.tr_tau : nullptr;
    A.pvc = h->has_pvc ? ep.pvc : nullptr;
    A.reinit = h->reinit ? 1 : 0;
    A.vol = h->reinit ? nullptr : a->tvol;
    A.mass = h->reinit ? nullptr : ep.mass;
    A.psize = h->reinit ? nullptr : ep.psize;
    A.vsc = a->tvsc;
    A.fn_off = h->d_fn_off;
    A.fn_x = h->d_fn_x;
    A.fn_y = h->d_fn_y;
    A.step = (int)a->seg_first;
    const float** tp[NTP] = {&A.x, &A.y, &A.vx, &A.vy, &A.sxx, &A.syy, &A.szz, &A.sxy, &A.rho};
    for (int k = 0; k < NTP; ++k) *tp[k] = a->tp[k];
    A.cflag = a->tflag;
    const float** tn[NTN] = {&A.nm, &A.nvax, &A.nvay, &A.nvbx, &A.nvby, &A.nax, &A.nay};
    for (int k = 0; k < NTN; ++k) *tn[k] = a->tn[k];
    float** lam[NLAM] = {&A.lx, &A.ly, &A.lvx, &A.lvy, &A.lsxx, &A.lsyy, &A.lszz, &A.lsxy,
                         &A.lrho, &A.lE, &A.lvol, &A.lvsc};
    for (int k = 0; k < NLAM; ++k) *lam[k] = a->lam[k];
    float** ps[NPS] = {&A.r0b, &A.r1b, &A.r3b, &A.c0b, &A.c1b};
    for (int k = 0; k < NPS; ++k) *ps[k] = a->pscr[k];
    float** ns[NNS] = {&A.fbx, &A.fby, &A.mb, &A.vabx, &A.vaby, &A.qbx, &A.qby, &A.mbt};
    for (int k = 0; k < NNS; ++k) *ns[k] = a->nscr[k];
    A.cnt = a->cnt;
    A.sp = (long long)tape_stride(h);
    A.sn = h->nn;
    A.sc = h->ncell;
    return A;
}

// The tiles the reverse node passes visit: the forward step kernels' tiles of
// the segment's sort when the segment is one sort epoch (the classification
// of its re-run holds for every step; an empty tile's node adjoints and cell
// counts are read by no particle), else every tile.
void reverse_tiles(MpmHandle* h, AdjointState* a, const int4*& tiles, int& ntiles) {
    if (a->nep == 1) {
        tiles = h->step_tiles;
        ntiles = h->nact;
    } else {
        tiles = h->dtiles;
        ntiles = h->ntiles;
    }
}

int reverse_step(MpmHandle* h, AdjointState* a, int t, cudaStream_t s) {
    AdjStep A = base_args(h, a, a->epoch_of[t]);
    const size_t op = (size_t)t * A.sp, on = (size_t)t * A.sn, oc = (size_t)t * A.sc;
    A.x += op; A.y += op; A.vx += op; A.vy += op;
    A.sxx += op; A.syy += op; A.szz += op; A.sxy += op; A.rho += op;
    if (A.vol) A.vol += op;
    if (A.vsc) A.vsc += op;
    A.cflag += oc;
    A.nm += on; A.nvax += on; A.nvay += on; A.nvbx += on; A.nvby += on; A.nax += on; A.nay += on;
    A.step += t;
    const int4* tiles;
    int ntiles;
    reverse_tiles(h, a, tiles, ntiles);
    CK(h, launch_rev_step(A, h->usl, h->has_trac, tiles, ntiles, s));
    return MPM_OK;
}

// The reverse steps of a segment of `len` steps in one sort epoch as one
// graph (keyed by the length and the number of tiles it launches).
int reverse_graph(MpmHandle* h, AdjointState* a, int len, cudaStream_t s) {
    TRY(prepare_adj_graphs(h, a, s));
    const int4* tiles;
    int ntiles;
    reverse_tiles(h, a, tiles, ntiles);
    const int64_t key = (int64_t)len | ((int64_t)ntiles << 24);
    return run_cached_graph(h, a->g_rev, key, s, [&](cudaStream_t c) -> int {
        for (int t = len - 1; t >= 0; --t) TRY(reverse_step(h, a, t, c));
        return MPM_OK;
    });
}

// Zero the adjoint arrays; particle (n, 2) seeds in original order -> lam[0..3]
// in the storage order `pid`.  The zeros are one memset of the permutation
// scratch gathered into all NLAM arrays (two launches instead of NLAM).
// With wait == false the caller synchronises the stream before it returns
// (a host seed may be staged in h->stage: the copies and gathers are
// stream-ordered, so the second seed's copy follows the first one's gather).
int seed(MpmHandle* h, AdjointState* a, const float* dl_dloc, const float* dl_dvel,
         const int* pid, int on_device, cudaStream_t s, bool wait = true) {
    const int np = (int)h->np;
    CK(h, cudaMemsetAsync(a->lam_tmp, 0, sizeof(float) * NLAM * (size_t)np, s));
    CK(h, launch_gather_in(a->d_lam, NLAM, pid, np, a->lam_tmp, s));
    const float* src[2] = {dl_dloc, dl_dvel};
    for (int k = 0; k < 2; ++k) {
        if (!src[k]) continue;
        const void* d = nullptr;
        TRY(to_device(h, src[k], sizeof(float) * 2 * h->np, on_device, s, &d));
        CK(h, launch_gather_in(a->d_lam + 2 * k, 2, pid, np, static_cast<const float*>(d), s));
        if (wait) TRY(sync(h, s));
    }
    return MPM_OK;
}

// Adjoint arrays lam[first..] in storage order `pid` -> particle (n, ncomp)
// array in original order.  With wait == false the caller synchronises the
// stream before it returns (a host destination is written by an
// asynchronous copy out of h->stage, which the next emit reuses in stream
// order; a larger stage is allocated only after cudaFree has waited for the
// device).
int emit(MpmHandle* h, AdjointState* a, float* dst, int first, int ncomp, const int* pid,
         int on_device, cudaStream_t s, bool wait = true) {
    if (!dst) return MPM_OK;
    const size_t bytes = sizeof(float) * ncomp * h->np;
    float* d = dst;
    if (!on_device) {
        TRY(ensure_stage(h, bytes));
        d = static_cast<float*>(h->stage);
    }
    CK(h, launch_scatter_out(a->d_lam + first, ncomp, pid, (int)h->np, d, s));
    if (!on_device) CK(h, cudaMemcpyAsync(dst, d, bytes, cudaMemcpyDeviceToHost, s));
    return wait ? sync(h, s) : MPM_OK;
}

int emit_all(MpmHandle* h, AdjointState* a, float* dl_dE, float* dl_dloc0, float* dl_dvel0,
             int on_device, cudaStream_t s, bool wait = true) {
    const int* pid = a->epochs[0].pid;   // the order of the first checkpoint
    TRY(emit(h, a, dl_dE, 9, 1, pid, on_device, s, wait));
    TRY(emit(h, a, dl_dloc0, 0, 2, pid, on_device, s, wait));
    return emit(h, a, dl_dvel0, 2, 2, pid, on_device, s, wait);
}

int check_supported(MpmHandle* h) {
    if (h->ndim != 2) return fail(h, MPM_ERR_UNSUPPORTED, "the adjoint implements Quadrilateral4Node meshes");
    return MPM_OK;
}

// Start a recording on h: checks, state and bookkeeping.
int record_begin(MpmHandle* h, int nsteps, int K) {
    if (!h->initialized) return fail(h, MPM_ERR_STATE, "initialize first");
    if (nsteps < 1 || K < 1) return fail(h, MPM_ERR_INVALID, "nsteps and checkpoint_steps must be >= 1");
    if (h->np <= 0) return fail(h, MPM_ERR_STATE, "no particles");
    TRY(check_supported(h));
    if (!h->adj) h->adj = new AdjointState();
    AdjointState* a = h->adj;
    fit(h, a);
    a->valid = false;
    a->resort_steps.clear();
    a->step0 = h->step;
    a->K = K;
    a->nsteps = nsteps;
    a->nseg = (nsteps + K - 1) / K;
    a->recording = true;
    return MPM_OK;
}

void record_end(MpmHandle* h, bool ok) {
    AdjointState* a = h->adj;
    a->recording = false;
    if (!ok) return;
    std::sort(a->resort_steps.begin(), a->resort_steps.end());
    a->resort_steps.erase(std::unique(a->resort_steps.begin(), a->resort_steps.end()),
                          a->resort_steps.end());
    a->gen = h->gen;
    a->valid = true;
}

int check_recorded(MpmHandle* h) {
    AdjointState* a = h->adj;
    if (!a || !a->valid || a->np_alloc != h->np) return fail(h, MPM_ERR_STATE, "call mpm_record first");
    if (a->gen != h->gen) return fail(h, MPM_ERR_STATE, "the simulation changed since mpm_record");
    return MPM_OK;
}

}  // namespace

void adjoint_note_resort(MpmHandle* h) {
    if (h->adj && h->adj->recording) h->adj->resort_steps.push_back(h->step);
}

void adjoint_free(MpmHandle* h) {
    if (!h->adj) return;
    free_buffers(h, h->adj);
    delete h->adj;
    h->adj = nullptr;
}

void drop_batch_adj_graphs(BatchAdjoint* x) {
    for (auto& kv : x->g_rerun) cudaGraphExecDestroy(kv.second);
    for (auto& kv : x->g_rev) cudaGraphExecDestroy(kv.second);
    x->g_rerun.clear();
    x->g_rev.clear();
}

// The buffers and kernel builds the batched adjoint's graphs hold; the
// cached graphs are dropped when any of them changed.
void check_batch_adj_graphs(MpmBatch* b, BatchAdjoint* x) {
    const std::vector<uintptr_t> sig = {
        (uintptr_t)x->tape_p[0].segs, (uintptr_t)x->tape_p[0].blk, x->tape_p[0].nblocks,
        (uintptr_t)x->tape_p[1].segs, (uintptr_t)x->tape_p[1].blk, x->tape_p[1].nblocks,
        (uintptr_t)x->tape_n.segs, (uintptr_t)x->tape_n.blk, x->tape_n.nblocks,
        (uintptr_t)x->d_bases, (uintptr_t)x->d_table, (uintptr_t)x->part_blocks,
        (uintptr_t)x->n_part_blocks, (uintptr_t)b->d_tdescs, (uintptr_t)b->d_edescs,
        (uintptr_t)b->d_act_list, (uintptr_t)b->d_tiles, (uintptr_t)b->d_ctls,
        (uintptr_t)b->cfg.nk_ctas, (uintptr_t)b->cfg.g2p_ctas, (uintptr_t)b->cfg.forces_lpc};
    if (sig != x->gsig) {
        drop_batch_adj_graphs(x);
        x->gsig = sig;
    }
}

void batch_adjoint_free(MpmBatch* b) {
    BatchAdjoint* x = b->badj;
    if (!x) return;
    drop_batch_adj_graphs(x);
    cudaFree(x->d_bases);
    cudaFree(x->d_table);
    cudaFree(x->part_blocks);
    cudaFree(x->mismatch);
    if (x->h_mismatch) cudaFreeHost(x->h_mismatch);
    segbuf_free(x->tape_p[0]);
    segbuf_free(x->tape_p[1]);
    segbuf_free(x->tape_n);
    segbuf_free(x->misc);
    delete x;
    b->badj = nullptr;
}

}  // namespace mpm

using namespace mpm::batch;

namespace {

// Batched re-run of segment `seg` of every simulation (tape slots 0..len-1),
// with the bitwise check against the next checkpoints.
int batch_recompute(MpmBatch* b, BatchAdjoint* x, int seg, int len, cudaStream_t s) {
    const int n = (int)b->sims.size();
    std::vector<CopySeg> v;
    for (int i = 0; i < n; ++i) checkpoint_segments(b->sims[i], b->sims[i]->adj->ck[seg], false, v);
    BTRY(b, 0, run_segments(b->sims[0], x->misc, v, s));
    int r = read_statuses(b, s);   // (clears the restored status words)
    if (r != MPM_OK) return r;
    v.clear();
    for (int i = 0; i < n; ++i) {
        AdjointState* a = b->sims[i]->adj;
        a->epoch_of.assign(len, 0);
        a->nep = 0;
        BTRY(b, i, epoch_segments(b->sims[i], a, 0, v));
        a->nep = 1;
    }
    BTRY(b, 0, run_segments(b->sims[0], x->misc, v, s));
    // tape tables: particle copies for even and odd t (each simulation's own
    // parity), nodal copies
    auto build_particle_tables = [&]() -> int {
        for (int q = 0; q < 2; ++q) {
            std::vector<CopySeg> w;
            for (MpmHandle* h : b->sims)
                tape_particle_segments(h, h->adj, (int)((h->step + q) & 1), w);
            BTRY(b, 0, upload_segments(b->sims[0], x->tape_p[q], w, s));
        }
        return MPM_OK;
    };
    // (the parity of slot t is that of the segment's first step plus t)
    std::vector<int64_t> first(n);
    for (int i = 0; i < n; ++i) {
        first[i] = b->sims[i]->step;
        b->sims[i]->adj->seg_first = first[i];
    }
    r = build_particle_tables();
    if (r != MPM_OK) return r;
    v.clear();
    for (MpmHandle* h : b->sims) tape_node_segments(h, h->adj, v);
    BTRY(b, 0, upload_segments(b->sims[0], x->tape_n, v, s));
    bool resorts = false;
    for (int i = 0; i < n && !resorts; ++i)
        for (int t = 0; t < len && !resorts; ++t) resorts = resorts_at(b->sims[i]->adj, first[i] + t);
    if (!resorts) {
        // one sort epoch for every simulation: the segment's steps with their
        // tape copies as one graph (the same launches as the loop below)
        r = prepare_tiles(b, s);
        if (r != MPM_OK) return r;
        check_batch_adj_graphs(b, x);
        const int64_t key = (int64_t)len | ((int64_t)b->nact << 20) | ((int64_t)b->nemp << 42);
        BTRY(b, 0, run_cached_graph(b->sims[0], x->g_rerun, key, s, [&](cudaStream_t c) -> int {
            for (int t = 0; t < len; ++t) {
                const SegBuf& tp = x->tape_p[t & 1];
                CK(b->sims[0], launch_copy_segments(tp.blk, tp.nblocks, t, c));
                const int rr = launch_batch_steps(b, 1, c);
                if (rr != MPM_OK) return fail(b->sims[0], MPM_ERR_CUDA, "%s", b->err.c_str());
                CK(b->sims[0], launch_copy_segments(x->tape_n.blk, x->tape_n.nblocks, t, c));
            }
            return MPM_OK;
        }));
        for (MpmHandle* h : b->sims) h->step += len;
    }
    for (int t = 0; t < len && resorts; ++t) {
        bool resorted = false;
        for (int i = 0; i < n; ++i) {
            MpmHandle* h = b->sims[i];
            if (!resorts_at(h->adj, first[i] + t)) continue;
            BTRY(b, i, resort(h, s));
            BTRY(b, i, capture_epoch(h, h->adj, s));
            resorted = true;
        }
        if (resorted) {
            // tables are built for the parity at t = 0: shift the simulations' steps back
            for (int i = 0; i < n; ++i) b->sims[i]->step -= t;
            r = build_particle_tables();
            for (int i = 0; i < n; ++i) b->sims[i]->step += t;
            if (r != MPM_OK) return r;
        }
        const SegBuf& tp = x->tape_p[t & 1];
        BCK(b, launch_copy_segments(tp.blk, tp.nblocks, t, s));
        // the tile records hold the sort: refreshed at the segment start and
        // after a re-sort only
        if (t == 0 || resorted) {
            r = prepare_tiles(b, s);
            if (r != MPM_OK) return r;
        }
        r = launch_batch_steps(b, 1, s);
        if (r != MPM_OK) return r;
        for (MpmHandle* h : b->sims) h->step++;
        BCK(b, launch_copy_segments(x->tape_n.blk, x->tape_n.nblocks, t, s));
        for (MpmHandle* h : b->sims) h->adj->epoch_of[t] = h->adj->nep - 1;
    }
    r = read_statuses(b, s);
    if (r != MPM_OK) return r;
    v.clear();
    for (int i = 0; i < n; ++i) {
        const int st = b->h_status[i].status;
        if (st & (ST_DRIFT_VIOLATION | ST_OUT_OF_MESH))
            return bfail(b, MPM_ERR_STATE, "simulation %d: re-run of segment %d left the recorded run",
                         i, seg);
        if (b->sims[i]->step != b->sims[i]->adj->ck[seg + 1].step)
            return bfail(b, MPM_ERR_STATE, "simulation %d: step count of the re-run differs", i);
        check_segments(b->sims[i], b->sims[i]->adj, seg, v);
    }
    BTRY(b, 0, upload_segments(b->sims[0], x->misc, v, s));
    BCK(b, cudaMemsetAsync(x->mismatch, 0, sizeof(int), s));
    BCK(b, launch_compare_segments(x->misc.blk, x->misc.nblocks,
                                   x->mismatch, s));
    BCK(b, cudaMemcpyAsync(x->h_mismatch, x->mismatch, sizeof(int), cudaMemcpyDeviceToHost, s));
    BCK(b, cudaStreamSynchronize(s));
    if (*x->h_mismatch != 0)
        return bfail(b, MPM_ERR_STATE, "re-run of segment %d did not reproduce the recorded run "
                     "(%d words differ)", seg, *x->h_mismatch);
    return MPM_OK;
}

int ensure_batch_adjoint(MpmBatch* b, cudaStream_t s) {
    if (!b->badj) b->badj = new BatchAdjoint();
    BatchAdjoint* x = b->badj;
    const int n = (int)b->sims.size();
    if (!x->d_bases) {
        BCK(b, cudaMalloc(&x->d_bases, sizeof(AdjStep) * n));
        BCK(b, cudaMalloc(&x->d_table, sizeof(AdjStep) * n));
        BCK(b, cudaMalloc(&x->mismatch, sizeof(int)));
        BCK(b, cudaMallocHost(&x->h_mismatch, sizeof(int)));
    }
    // block maps (particle counts may have changed since the last call)
    std::vector<int2> pb;
    for (int i = 0; i < n; ++i) {
        const MpmHandle* h = b->sims[i];
        for (int c = 0; c * ADJ_BLOCK * ADJ_ITER < h->np; ++c) pb.push_back(make_int2(i, c));
    }
    cudaFree(x->part_blocks);
    x->part_blocks = nullptr;
    BCK(b, cudaMalloc(&x->part_blocks, sizeof(int2) * pb.size()));
    BCK(b, cudaMemcpyAsync(x->part_blocks, pb.data(), sizeof(int2) * pb.size(), cudaMemcpyHostToDevice, s));
    BCK(b, cudaStreamSynchronize(s));
    x->n_part_blocks = (int)pb.size();
    return MPM_OK;
}

}  // namespace

extern "C" {

int mpm_record(MpmHandle* h, int nsteps, int checkpoint_steps, void* stream) {
    if (!h) return MPM_ERR_INVALID;
    if (h->ndim == 1) return line_record(h, nsteps, S(stream));   // full tape, no checkpoints
    TRY(record_begin(h, nsteps, checkpoint_steps));
    cudaStream_t s = S(stream);
    AdjointState* a = h->adj;
    int r = MPM_OK;
    for (int seg = 0; seg < a->nseg && r == MPM_OK; ++seg) {
        std::vector<CopySeg> v;
        r = save_checkpoint(h, a, seg, v);
        if (r == MPM_OK) r = run_segments(h, h->segbuf, v, s);
        const int len = std::min(checkpoint_steps, nsteps - seg * checkpoint_steps);
        if (r == MPM_OK) r = mpm_step(h, len, stream);
    }
    if (r == MPM_OK) {
        std::vector<CopySeg> v;
        r = save_checkpoint(h, a, a->nseg, v);
        if (r == MPM_OK) r = run_segments(h, h->segbuf, v, s);
        if (r == MPM_OK) r = sync(h, s);
    }
    record_end(h, r == MPM_OK);
    return r;
}

int mpm_adjoint(MpmHandle* h, const float* dl_dloc, const float* dl_dvel, float* dl_dE,
                float* dl_dloc0, float* dl_dvel0, int on_device, void* stream) {
    if (!h) return MPM_ERR_INVALID;
    if (h->ndim == 1)
        return line_adjoint(h, dl_dloc, dl_dvel, dl_dE, dl_dloc0, dl_dvel0, on_device, S(stream));
    TRY(check_recorded(h));
    if (!dl_dloc) return fail(h, MPM_ERR_INVALID, "dl_dloc is null");
    AdjointState* a = h->adj;
    cudaStream_t s = S(stream);
    const int K = a->K;
    TRY(ensure_adjoint_buffers(h, a, K, s));
    // the seeds are in the order of the recorded end state (the current one)
    TRY(seed(h, a, dl_dloc, dl_dvel, h->ps[h->pcur].pid, on_device, s));
    int r = MPM_OK;
    for (int seg = a->nseg - 1; seg >= 0 && r == MPM_OK; --seg) {
        const int len = (int)std::min<int64_t>(K, a->nsteps - (int64_t)seg * K);
        r = recompute_segment(h, a, seg, len, s);
        // one sort epoch: the segment's reverse steps as a graph (tractions
        // need the step number, which the graph would hold by value)
        if (r == MPM_OK && a->nep == 1 && !h->has_trac) {
            r = reverse_graph(h, a, len, s);
            continue;
        }
        for (int t = len - 1; t >= 0 && r == MPM_OK; --t) {
            if (t < len - 1 && a->epoch_of[t] != a->epoch_of[t + 1])
                r = permute(h, a, a->epochs[a->epoch_of[t + 1]].pid, a->epochs[a->epoch_of[t]].pid, s);
            if (r == MPM_OK) r = reverse_step(h, a, t, s);
        }
        if (r == MPM_OK && a->epoch_of[0] != 0)
            r = permute(h, a, a->epochs[a->epoch_of[0]].pid, a->epochs[0].pid, s);
    }
    if (r == MPM_OK) r = emit_all(h, a, dl_dE, dl_dloc0, dl_dvel0, on_device, s);
    // leave the handle at the recorded end state
    const int r2 = restore_checkpoint(h, a->ck[a->nseg], s);
    TRY(r);
    return r2;
}

int mpm_batch_record(MpmBatch* b, int nsteps, int checkpoint_steps, void* stream) {
    if (!b) return MPM_ERR_INVALID;
    int r = check_ready(b);
    if (r != MPM_OK) return r;
    const int n = (int)b->sims.size();
    for (int i = 0; i < n; ++i) BTRY(b, i, record_begin(b->sims[i], nsteps, checkpoint_steps));
    cudaStream_t s = S(stream);
    const int nseg = b->sims[0]->adj->nseg;
    for (int seg = 0; seg <= nseg && r == MPM_OK; ++seg) {
        std::vector<CopySeg> v;
        for (int i = 0; i < n && r == MPM_OK; ++i) {
            r = save_checkpoint(b->sims[i], b->sims[i]->adj, seg, v);
            if (r != MPM_OK) r = from_sim(b, i, r);
        }
        if (r == MPM_OK && run_segments(b->sims[0], b->segbuf, v, s) != MPM_OK) r = from_sim(b, 0, MPM_ERR_CUDA);
        if (r == MPM_OK && seg < nseg)
            r = batch_steps(b, std::min(checkpoint_steps, nsteps - seg * checkpoint_steps), s);
    }
    if (r == MPM_OK && cudaStreamSynchronize(s) != cudaSuccess) r = bfail(b, MPM_ERR_CUDA, "synchronise");
    for (MpmHandle* h : b->sims) record_end(h, r == MPM_OK);
    return r;
}

int mpm_batch_adjoint(MpmBatch* b, const float* const* dl_dloc, const float* const* dl_dvel,
                      float* const* dl_dE, float* const* dl_dloc0, float* const* dl_dvel0,
                      int on_device, void* stream) {
    if (!b) return MPM_ERR_INVALID;
    if (!dl_dloc) return bfail(b, MPM_ERR_INVALID, "dl_dloc is null");
    const int n = (int)b->sims.size();
    for (int i = 0; i < n; ++i) {
        MpmHandle* h = b->sims[i];
        BTRY(b, i, check_recorded(h));
        if (h->adj->nsteps != b->sims[0]->adj->nsteps || h->adj->K != b->sims[0]->adj->K)
            return bfail(b, MPM_ERR_STATE, "simulation %d was recorded apart from the batch", i);
        if (!dl_dloc[i]) return bfail(b, MPM_ERR_INVALID, "dl_dloc[%d] is null", i);
    }
    cudaStream_t s = S(stream);
    const int K = b->sims[0]->adj->K, nseg = b->sims[0]->adj->nseg;
    const int64_t nsteps = b->sims[0]->adj->nsteps;
    int r = ensure_batch_adjoint(b, s);
    if (r != MPM_OK) return r;
    BatchAdjoint* x = b->badj;
    for (int i = 0; i < n; ++i) BTRY(b, i, ensure_adjoint_buffers(b->sims[i], b->sims[i]->adj, K, s));
    for (int i = 0; i < n; ++i) {
        MpmHandle* h = b->sims[i];
        // (no wait per simulation: the segment loop synchronises the stream,
        // and a failure here waits for the seeds already in flight)
        const int e = seed(h, h->adj, dl_dloc[i], dl_dvel ? dl_dvel[i] : nullptr, h->ps[h->pcur].pid,
                           on_device, s, false);
        if (e != MPM_OK) {
            cudaStreamSynchronize(s);
            return from_sim(b, i, e);
        }
    }
    x->bases.assign(n, AdjStep{});
    std::vector<int> cur(n, -1);   // epoch whose pointers bases[i] holds
    bool any_pvc = false, any_newt = false;
    for (MpmHandle* h : b->sims) {
        any_pvc = any_pvc || h->has_pvc;
        any_newt = any_newt || h->adj->tvsc != nullptr;
    }
    for (int seg = nseg - 1; seg >= 0 && r == MPM_OK; --seg) {
        const int len = (int)std::min<int64_t>(K, nsteps - (int64_t)seg * K);
        r = batch_recompute(b, x, seg, len, s);
        if (r != MPM_OK) break;
        for (int i = 0; i < n; ++i) {
            AdjointState* a = b->sims[i]->adj;
            x->bases[i] = base_args(b->sims[i], a, a->epoch_of[len - 1]);
            cur[i] = a->epoch_of[len - 1];
        }
        BCK(b, cudaMemcpyAsync(x->d_bases, x->bases.data(), sizeof(AdjStep) * n, cudaMemcpyHostToDevice, s));
        // the reverse node passes visit the active tiles of the re-run's
        // classification when no simulation re-sorted in the segment (see
        // reverse_tiles), else every tile
        bool one_epoch = true;
        for (MpmHandle* h : b->sims) one_epoch = one_epoch && h->adj->nep == 1;
        const int4* rtiles = one_epoch ? b->d_act_list : b->d_tiles;
        const int nrtiles = one_epoch ? b->nact : b->ntiles;
        if (one_epoch) {
            // no permutation between steps: the segment's reverse steps as one graph
            check_batch_adj_graphs(b, x);
            const int64_t key = (int64_t)len | ((int64_t)nrtiles << 20) | ((int64_t)x->n_part_blocks << 42);
            r = run_cached_graph(b->sims[0], x->g_rev, key, s, [&](cudaStream_t c) -> int {
                for (int t = len - 1; t >= 0; --t) {
                    CK(b->sims[0], launch_adj_table(x->d_bases, n, t, x->d_table, c));
                    CK(b->sims[0], launch_rev_batch(x->d_table, b->cfg.usl, b->cfg.traction, any_pvc,
                                                    b->cfg.reinit, any_newt, rtiles, nrtiles, x->part_blocks,
                                                    x->n_part_blocks, c));
                }
                return MPM_OK;
            });
            if (r != MPM_OK) r = from_sim(b, 0, r);
        }
        for (int t = len - 1; t >= 0 && r == MPM_OK && !one_epoch; --t) {
            for (int i = 0; i < n && r == MPM_OK; ++i) {
                MpmHandle* h = b->sims[i];
                AdjointState* a = h->adj;
                if (a->epoch_of[t] == cur[i]) continue;
                r = permute(h, a, a->epochs[cur[i]].pid, a->epochs[a->epoch_of[t]].pid, s);
                if (r != MPM_OK) {
                    r = from_sim(b, i, r);
                    break;
                }
                cur[i] = a->epoch_of[t];
                x->bases[i] = base_args(h, a, cur[i]);
                if (cudaMemcpyAsync(x->d_bases + i, &x->bases[i], sizeof(AdjStep), cudaMemcpyHostToDevice,
                                    s) != cudaSuccess)
                    r = bfail(b, MPM_ERR_CUDA, "argument upload");
            }
            if (r != MPM_OK) break;
            BCK(b, launch_adj_table(x->d_bases, n, t, x->d_table, s));
            BCK(b, launch_rev_batch(x->d_table, b->cfg.usl, b->cfg.traction, any_pvc, b->cfg.reinit,
                                    any_newt, rtiles, nrtiles, x->part_blocks, x->n_part_blocks, s));
        }
        for (int i = 0; i < n && r == MPM_OK; ++i) {
            MpmHandle* h = b->sims[i];
            AdjointState* a = h->adj;
            if (a->epoch_of[0] != 0) {
                const int e = permute(h, a, a->epochs[a->epoch_of[0]].pid, a->epochs[0].pid, s);
                if (e != MPM_OK) r = from_sim(b, i, e);
            }
        }
        // (the host copy of the arguments must outlive the uploads)
        if (r == MPM_OK && cudaStreamSynchronize(s) != cudaSuccess) r = bfail(b, MPM_ERR_CUDA, "synchronise");
    }
    for (int i = 0; i < n && r == MPM_OK; ++i) {
        MpmHandle* h = b->sims[i];
        const int e = emit_all(h, h->adj, dl_dE ? dl_dE[i] : nullptr, dl_dloc0 ? dl_dloc0[i] : nullptr,
                               dl_dvel0 ? dl_dvel0[i] : nullptr, on_device, s, false);
        if (e != MPM_OK) r = from_sim(b, i, e);
    }
    // leave every simulation at the recorded end state (read_statuses
    // synchronises the stream: the gradients' copies are complete on return)
    std::vector<CopySeg> v;
    for (MpmHandle* h : b->sims) checkpoint_segments(h, h->adj->ck[nseg], false, v);
    int r2 = run_segments(b->sims[0], x->misc, v, s);
    if (r2 == MPM_OK) {
        r2 = read_statuses(b, s);
    } else {
        cudaStreamSynchronize(s);
        r2 = from_sim(b, 0, r2);
    }
    if (r != MPM_OK) return r;
    return r2;
}

}  // extern "C"
