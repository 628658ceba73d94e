// Differentiation of the explicit step: a checkpointed forward run
// (mpm_record) and the hand-written discrete adjoint (mpm_adjoint).
//
// mpm_record advances like mpm_step and keeps a full copy of the simulation
// state at the start of every segment of K steps (and at the end), plus the
// steps before which the particles were re-sorted.  mpm_adjoint walks the
// segments backwards: it restores the segment's checkpoint, re-runs its K
// steps one at a time while copying each step's start state and nodal results
// into a tape (re-sorting at the recorded steps, so the storage order of every
// step matches the recorded run), then runs the four reverse passes of
// mpm_adjoint.h for each step from the last to the first.  The adjoint arrays
// follow the storage order of the step being reversed; where a re-sort
// separates two steps they are permuted through the original particle order.
// Memory: one checkpoint per segment (the particle state, cell starts and
// persistent nodal velocity) and a tape of K steps (9 floats per particle, 7
// per node and 1 byte per cell per step).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "mpm_adjoint.h"
#include "mpm_handle.h"

using namespace mpm;
using namespace mpm::host;

namespace mpm {

namespace {

constexpr int NLAM = 10;   // adjoint arrays: x y vx vy sxx syy szz sxy rho E
constexpr int NTP = 9;     // tape per particle: x y vx vy sxx syy szz sxy rho
constexpr int NTN = 7;     // tape per node: m vAx vAy vBx vBy aBx aBy
constexpr int NPS = 5;     // per-particle scratch: r0b r1b r3b c0b c1b
constexpr int NNS = 8;     // per-node scratch: fbx fby mb vabx vaby qbx qby mbt

struct Epoch {               // arrays of one sort epoch inside a segment
    int* pid = nullptr;
    uint8_t* mat = nullptr;
    float* E = nullptr;
    int* cstart = nullptr;
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
    uint8_t* tflag = nullptr;
    float* tn[NTN] = {};
    std::vector<Epoch> epochs;
    std::vector<int> epoch_of;
    float* lam[NLAM] = {};
    float* lam_tmp = nullptr;
    int* lam_pid = nullptr;
    float** d_lam = nullptr;
    float* pscr[NPS] = {};
    float* nscr[NNS] = {};
    int* cnt = nullptr;
    int* mismatch = nullptr;   // device counter of the re-run check
    int* h_mismatch = nullptr; // pinned
};

namespace {

void free_buffers(MpmHandle* h, AdjointState* a) {
    for (auto& c : a->ck) checkpoint_free(h, c);
    a->ck.clear();
    for (float*& p : a->tp) { dfree(h, p); p = nullptr; }
    for (float*& p : a->tn) { dfree(h, p); p = nullptr; }
    dfree(h, a->tflag);
    a->tflag = nullptr;
    a->tape_slots = 0;
    for (Epoch& e : a->epochs) {
        dfree(h, e.pid);
        dfree(h, e.mat);
        dfree(h, e.E);
        dfree(h, e.cstart);
    }
    a->epochs.clear();
    for (float*& p : a->lam) { dfree(h, p); p = nullptr; }
    for (float*& p : a->pscr) { dfree(h, p); p = nullptr; }
    for (float*& p : a->nscr) { dfree(h, p); p = nullptr; }
    dfree(h, a->lam_tmp);
    dfree(h, a->lam_pid);
    dfree(h, a->d_lam);
    dfree(h, a->cnt);
    dfree(h, a->mismatch);
    if (a->h_mismatch) cudaFreeHost(a->h_mismatch);
    a->mismatch = nullptr;
    a->h_mismatch = nullptr;
    a->lam_tmp = nullptr;
    a->lam_pid = nullptr;
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

int save_checkpoint(MpmHandle* h, AdjointState* a, size_t idx, cudaStream_t s) {
    if (a->ck.size() <= idx) a->ck.resize(idx + 1);
    Checkpoint& c = a->ck[idx];
    TRY(checkpoint_alloc(h, c));
    std::vector<CopySeg> v;
    checkpoint_segments(h, c, true, v);
    return run_segments(h, h->segbuf, v, s);
}

int restore_checkpoint(MpmHandle* h, Checkpoint& c, cudaStream_t s) {
    std::vector<CopySeg> v;
    checkpoint_segments(h, c, false, v);
    TRY(run_segments(h, h->segbuf, v, s));
    TRY(clear_status(h, s));
    return sync(h, s);
}

int ensure_adjoint_buffers(MpmHandle* h, AdjointState* a, int slots, cudaStream_t s) {
    const size_t np = (size_t)h->np, nn = (size_t)h->nn;
    if (a->tape_slots < slots) {
        for (float*& p : a->tp) { dfree(h, p); p = nullptr; }
        for (float*& p : a->tn) { dfree(h, p); p = nullptr; }
        dfree(h, a->tflag);
        a->tflag = nullptr;
        a->tape_slots = 0;
        for (float*& p : a->tp) TRY(dalloc(h, &p, np * slots));
        for (float*& p : a->tn) TRY(dalloc(h, &p, nn * slots));
        TRY(dalloc(h, &a->tflag, (size_t)h->ncell * slots));
        a->tape_slots = slots;
    }
    if (!a->lam[0]) {
        for (float*& p : a->lam) TRY(dalloc(h, &p, np));
        for (float*& p : a->pscr) TRY(dalloc(h, &p, np));
        for (float*& p : a->nscr) TRY(dalloc(h, &p, nn));
        TRY(dalloc(h, &a->lam_tmp, np * NLAM));
        TRY(dalloc(h, &a->lam_pid, np));
        TRY(dalloc(h, &a->d_lam, NLAM));
        TRY(dalloc(h, &a->cnt, (size_t)h->ncell));
        TRY(dalloc(h, &a->mismatch, 1));
        CK(h, cudaMallocHost(&a->h_mismatch, sizeof(int)));
        CK(h, cudaMemcpyAsync(a->d_lam, a->lam, sizeof(float*) * NLAM, cudaMemcpyHostToDevice, s));
        TRY(sync(h, s));
    }
    return MPM_OK;
}

// Copy the current sort epoch's order-dependent arrays into epoch slot e.
int capture_epoch(MpmHandle* h, AdjointState* a, size_t e, cudaStream_t s) {
    const size_t np = (size_t)h->np;
    if (a->epochs.size() <= e) {
        Epoch ep;
        TRY(dalloc(h, &ep.pid, np));
        TRY(dalloc(h, &ep.mat, np));
        if (h->has_E) TRY(dalloc(h, &ep.E, np));
        TRY(dalloc(h, &ep.cstart, (size_t)h->ncell + 2));
        a->epochs.push_back(ep);
    }
    Epoch& ep = a->epochs[e];
    if (h->has_E && !ep.E) TRY(dalloc(h, &ep.E, np));
    const PSet& p = h->ps[h->pcur];
    CK(h, cudaMemcpyAsync(ep.pid, p.pid, sizeof(int) * np, cudaMemcpyDeviceToDevice, s));
    CK(h, cudaMemcpyAsync(ep.mat, p.mat, np, cudaMemcpyDeviceToDevice, s));
    if (h->has_E) CK(h, cudaMemcpyAsync(ep.E, p.E, sizeof(float) * np, cudaMemcpyDeviceToDevice, s));
    CK(h, cudaMemcpyAsync(ep.cstart, h->cstart[h->cs_cur], sizeof(int) * (h->ncell + 2),
                          cudaMemcpyDeviceToDevice, s));
    return MPM_OK;
}

// Re-run segment `seg` from its checkpoint, filling tape slots 0..len-1.
int recompute_segment(MpmHandle* h, AdjointState* a, int seg, int len, cudaStream_t s) {
    TRY(restore_checkpoint(h, a->ck[seg], s));
    TRY(clear_status(h, s));
    const int64_t first = a->ck[seg].step;
    const size_t np = (size_t)h->np, nn = (size_t)h->nn;
    a->epoch_of.assign(len, 0);
    int nep = 0;
    TRY(capture_epoch(h, a, nep++, s));
    for (int t = 0; t < len; ++t) {
        if (std::binary_search(a->resort_steps.begin(), a->resort_steps.end(), first + t)) {
            TRY(resort(h, s));
            TRY(capture_epoch(h, a, nep++, s));
        }
        const PSet& p = h->ps[h->pcur];
        const int par = parity(h);
        CopyJob jp{};
        const float* src[NTP] = {p.x, p.y, p.vx, p.vy, p.sxx[par], p.syy[par], p.szz[par],
                                 p.sxy[par], p.rho[par]};
        for (int k = 0; k < NTP; ++k) {
            jp.src[k] = src[k];
            jp.dst[k] = a->tp[k] + np * t;
        }
        jp.count = NTP;
        jp.n = (int)np;
        CK(h, launch_copy_f32(jp, s));
        CK(h, cudaMemcpyAsync(a->tflag + (size_t)h->ncell * t, h->cflag, h->ncell,
                              cudaMemcpyDeviceToDevice, s));
        TRY(launch_steps(h, 1, s));
        h->step++;
        CopyJob jn{};
        const float* nsrc[NTN] = {h->nm, h->nvax, h->nvay, h->nvbx, h->nvby, h->nax, h->nay};
        for (int k = 0; k < NTN; ++k) {
            jn.src[k] = nsrc[k];
            jn.dst[k] = a->tn[k] + nn * t;
        }
        jn.count = NTN;
        jn.n = (int)nn;
        CK(h, launch_copy_f32(jn, s));
        a->epoch_of[t] = nep - 1;
    }
    TRY(read_ctl(h, s));
    int st = 0;
    TRY(check_status(h, st));
    // the re-run must end bit for bit in the recorded state of the next checkpoint
    const Checkpoint& next = a->ck[seg + 1];
    std::vector<float**> f = movable_f32(h, h->ps[h->pcur], false);
    CK(h, cudaMemsetAsync(a->mismatch, 0, sizeof(int), s));
    for (size_t i = 0; i < f.size(); ++i)
        CK(h, launch_count_mismatch(*f[i], next.f[i], (int)np, a->mismatch, s));
    CK(h, cudaMemcpyAsync(a->h_mismatch, a->mismatch, sizeof(int), cudaMemcpyDeviceToHost, s));
    TRY(sync(h, s));
    if ((st & ST_DRIFT_VIOLATION) || *a->h_mismatch != 0 || h->step != next.step)
        return fail(h, MPM_ERR_STATE,
                    "re-run of steps %lld..%lld did not reproduce the recorded run (%d values differ)",
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

AdjStep step_args(MpmHandle* h, AdjointState* a, int t) {
    const size_t np = (size_t)h->np, nn = (size_t)h->nn;
    const Epoch& ep = a->epochs[a->epoch_of[t]];
    AdjStep A{};
    A.nx = h->nx;
    A.ny = h->ny;
    A.np = (int)np;
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
    const float** tp[NTP] = {&A.x, &A.y, &A.vx, &A.vy, &A.sxx, &A.syy, &A.szz, &A.sxy, &A.rho};
    for (int k = 0; k < NTP; ++k) *tp[k] = a->tp[k] + np * t;
    A.cflag = a->tflag + (size_t)h->ncell * t;
    const float** tn[NTN] = {&A.nm, &A.nvax, &A.nvay, &A.nvbx, &A.nvby, &A.nax, &A.nay};
    for (int k = 0; k < NTN; ++k) *tn[k] = a->tn[k] + nn * t;
    float** lam[NLAM] = {&A.lx, &A.ly, &A.lvx, &A.lvy, &A.lsxx, &A.lsyy, &A.lszz, &A.lsxy,
                         &A.lrho, &A.lE};
    for (int k = 0; k < NLAM; ++k) *lam[k] = a->lam[k];
    float** ps[NPS] = {&A.r0b, &A.r1b, &A.r3b, &A.c0b, &A.c1b};
    for (int k = 0; k < NPS; ++k) *ps[k] = a->pscr[k];
    float** ns[NNS] = {&A.fbx, &A.fby, &A.mb, &A.vabx, &A.vaby, &A.qbx, &A.qby, &A.mbt};
    for (int k = 0; k < NNS; ++k) *ns[k] = a->nscr[k];
    A.cnt = a->cnt;
    return A;
}

int reverse_step(MpmHandle* h, AdjointState* a, int t, cudaStream_t s) {
    const AdjStep A = step_args(h, a, t);
    CK(h, launch_rev_nodal_update(A, s));
    CK(h, launch_rev_forces(A, s));
    CK(h, launch_rev_nodal_kinematics(A, s));
    CK(h, launch_rev_mass_momentum(A, s));
    return MPM_OK;
}

// Particle (n, ncomp) array in original order -> adjoint arrays lam[first..].
int seed(MpmHandle* h, AdjointState* a, const float* src, int first, int ncomp, int on_device,
         cudaStream_t s) {
    const void* d = nullptr;
    TRY(to_device(h, src, sizeof(float) * ncomp * h->np, on_device, s, &d));
    CK(h, launch_gather_in(a->d_lam + first, ncomp, a->lam_pid, (int)h->np,
                           static_cast<const float*>(d), s));
    return sync(h, s);
}

// Adjoint arrays lam[first..] -> particle (n, ncomp) array in original order.
int emit(MpmHandle* h, AdjointState* a, float* dst, int first, int ncomp, int on_device,
         cudaStream_t s) {
    const size_t bytes = sizeof(float) * ncomp * h->np;
    float* d = dst;
    if (!on_device) {
        TRY(ensure_stage(h, bytes));
        d = static_cast<float*>(h->stage);
    }
    CK(h, launch_scatter_out(a->d_lam + first, ncomp, a->lam_pid, (int)h->np, d, s));
    if (!on_device) CK(h, cudaMemcpyAsync(dst, d, bytes, cudaMemcpyDeviceToHost, s));
    return sync(h, s);
}

int check_supported(MpmHandle* h) {
    if (h->usl) return fail(h, MPM_ERR_UNSUPPORTED, "the adjoint implements the USF scheme");
    if (!h->reinit)
        return fail(h, MPM_ERR_UNSUPPORTED,
                    "the adjoint implements the per-step volume set-up of solve_jit");
    if (h->has_trac) return fail(h, MPM_ERR_UNSUPPORTED, "the adjoint does not cover particle tractions");
    for (const MatDev& m : h->mats)
        if (m.type == MAT_NEWTONIAN)
            return fail(h, MPM_ERR_UNSUPPORTED, "the adjoint covers LinearElastic and SimpleMaterial");
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

}  // namespace mpm

extern "C" {

int mpm_record(MpmHandle* h, int nsteps, int checkpoint_steps, void* stream) {
    if (!h) return MPM_ERR_INVALID;
    if (!h->initialized) return fail(h, MPM_ERR_STATE, "initialize first");
    if (nsteps < 1 || checkpoint_steps < 1)
        return fail(h, MPM_ERR_INVALID, "nsteps and checkpoint_steps must be >= 1");
    if (h->np <= 0) return fail(h, MPM_ERR_STATE, "no particles");
    TRY(check_supported(h));
    cudaStream_t s = S(stream);
    if (!h->adj) h->adj = new AdjointState();
    AdjointState* a = h->adj;
    fit(h, a);
    a->valid = false;
    const int nseg = (nsteps + checkpoint_steps - 1) / checkpoint_steps;
    a->resort_steps.clear();
    a->step0 = h->step;
    a->K = checkpoint_steps;
    a->nsteps = nsteps;
    a->nseg = nseg;
    a->recording = true;
    int r = MPM_OK;
    for (int seg = 0; seg < nseg && r == MPM_OK; ++seg) {
        r = save_checkpoint(h, a, seg, s);
        const int len = std::min(checkpoint_steps, nsteps - seg * checkpoint_steps);
        if (r == MPM_OK) r = mpm_step(h, len, stream);
    }
    a->recording = false;
    TRY(r);
    TRY(save_checkpoint(h, a, nseg, s));
    std::sort(a->resort_steps.begin(), a->resort_steps.end());
    a->resort_steps.erase(std::unique(a->resort_steps.begin(), a->resort_steps.end()),
                          a->resort_steps.end());
    TRY(sync(h, s));
    a->gen = h->gen;
    a->valid = true;
    return MPM_OK;
}

int mpm_adjoint(MpmHandle* h, const float* dl_dloc, const float* dl_dvel, float* dl_dE,
                float* dl_dloc0, float* dl_dvel0, int on_device, void* stream) {
    if (!h) return MPM_ERR_INVALID;
    AdjointState* a = h->adj;
    if (!a || !a->valid || a->np_alloc != h->np)
        return fail(h, MPM_ERR_STATE, "call mpm_record first");
    if (a->gen != h->gen)
        return fail(h, MPM_ERR_STATE, "the simulation changed since mpm_record");
    if (!dl_dloc) return fail(h, MPM_ERR_INVALID, "dl_dloc is null");
    cudaStream_t s = S(stream);
    const int K = a->K;
    TRY(ensure_adjoint_buffers(h, a, K, s));
    for (float* p : a->lam) CK(h, cudaMemsetAsync(p, 0, sizeof(float) * h->np, s));
    CK(h, cudaMemcpyAsync(a->lam_pid, h->ps[h->pcur].pid, sizeof(int) * h->np,
                          cudaMemcpyDeviceToDevice, s));
    TRY(seed(h, a, dl_dloc, 0, 2, on_device, s));
    if (dl_dvel) TRY(seed(h, a, dl_dvel, 2, 2, on_device, s));

    int r = MPM_OK;
    for (int seg = a->nseg - 1; seg >= 0 && r == MPM_OK; --seg) {
        const int len = (int)std::min<int64_t>(K, a->nsteps - (int64_t)seg * K);
        r = recompute_segment(h, a, seg, len, s);
        if (r != MPM_OK) break;
        r = permute(h, a, a->lam_pid, a->epochs[a->epoch_of[len - 1]].pid, s);
        for (int t = len - 1; t >= 0 && r == MPM_OK; --t) {
            if (t < len - 1 && a->epoch_of[t] != a->epoch_of[t + 1])
                r = permute(h, a, a->epochs[a->epoch_of[t + 1]].pid, a->epochs[a->epoch_of[t]].pid, s);
            if (r == MPM_OK) r = reverse_step(h, a, t, s);
        }
        if (r == MPM_OK) {
            cudaError_t e = cudaMemcpyAsync(a->lam_pid, a->epochs[a->epoch_of[0]].pid,
                                            sizeof(int) * h->np, cudaMemcpyDeviceToDevice, s);
            if (e != cudaSuccess) r = fail(h, MPM_ERR_CUDA, "%s", cudaGetErrorString(e));
        }
    }
    if (r == MPM_OK && dl_dE) r = emit(h, a, dl_dE, 9, 1, on_device, s);
    if (r == MPM_OK && dl_dloc0) r = emit(h, a, dl_dloc0, 0, 2, on_device, s);
    if (r == MPM_OK && dl_dvel0) r = emit(h, a, dl_dvel0, 2, 2, on_device, s);
    // leave the handle at the recorded end state
    const int r2 = restore_checkpoint(h, a->ck[a->nseg], s);
    TRY(r);
    return r2;
}

}  // extern "C"
