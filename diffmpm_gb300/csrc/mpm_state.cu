// Whole-state copies of a simulation as lists of device-memory segments: the
// rollback snapshot of a step block and the checkpoints of the adjoint.  One
// launch copies a list, for one simulation or for every simulation of a batch.
#include <cuda_runtime.h>

#include <vector>

#include "mpm_handle.h"

namespace mpm {
namespace host {

namespace {

void add(std::vector<CopySeg>& out, const void* src, void* dst, size_t bytes, bool save) {
    if (!bytes) return;
    CopySeg s;
    s.src = save ? src : dst;
    s.dst = save ? dst : const_cast<void*>(src);
    s.bytes = bytes;
    s.dst_step = 0;
    out.push_back(s);
}

}  // namespace

void snapshot_segments(MpmHandle* h, bool save, std::vector<CopySeg>& out) {
    std::vector<float**> f = movable_f32(h, h->ps[h->pcur], true);
    const size_t np = (size_t)h->np;
    for (size_t i = 0; i < f.size(); ++i) add(out, *f[i], h->snap_f[i], sizeof(float) * np, save);
    add(out, h->cflag, h->snap_cflag, (size_t)h->ncell, save);
    add(out, h->nvbx, h->snap_nvbx, sizeof(float) * h->nn, save);
    add(out, h->nvby, h->snap_nvby, sizeof(float) * h->nn, save);
    add(out, h->ctl, h->snap_ctl, sizeof(Control), save);
}

int checkpoint_alloc(MpmHandle* h, Checkpoint& c) {
    const size_t np = (size_t)h->np;
    const size_t nf = movable_f32(h, h->ps[h->pcur], false).size();
    if (c.f.size() == nf && c.ctl && (!h->has_trac || c.tr_fn) && (!h->has_pvc || c.pvc)) return MPM_OK;
    checkpoint_free(h, c);
    c.f.assign(nf, nullptr);
    for (float*& p : c.f) TRY(dalloc(h, &p, np));
    TRY(dalloc(h, &c.mat, np));
    if (h->has_trac) {
        TRY(dalloc(h, &c.tr_fn, 2 * np));
        TRY(dalloc(h, &c.tr_tau, 2 * np));
    }
    if (h->has_pvc) TRY(dalloc(h, &c.pvc, 2 * np));
    TRY(dalloc(h, &c.cstart, (size_t)h->ncell + 2));
    TRY(dalloc(h, &c.cflag, (size_t)h->ncell));
    TRY(dalloc(h, &c.nvbx, (size_t)h->nn));
    TRY(dalloc(h, &c.nvby, (size_t)h->nn));
    TRY(dalloc(h, &c.ctl, 1));
    return MPM_OK;
}

void checkpoint_free(MpmHandle* h, Checkpoint& c) {
    for (float* p : c.f) dfree(h, p);
    dfree(h, c.mat);
    dfree(h, c.tr_fn);
    dfree(h, c.tr_tau);
    dfree(h, c.pvc);
    dfree(h, c.cstart);
    dfree(h, c.cflag);
    dfree(h, c.nvbx);
    dfree(h, c.nvby);
    dfree(h, c.ctl);
    c = Checkpoint{};
}

void checkpoint_segments(MpmHandle* h, Checkpoint& c, bool save, std::vector<CopySeg>& out) {
    if (save) {
        c.step = h->step;
        c.needs_resort = h->needs_resort;
    } else {
        h->step = c.step;
        h->needs_resort = c.needs_resort;
    }
    std::vector<float**> f = movable_f32(h, h->ps[h->pcur], false);
    const size_t np = (size_t)h->np;
    for (size_t i = 0; i < f.size(); ++i) add(out, *f[i], c.f[i], sizeof(float) * np, save);
    add(out, h->ps[h->pcur].mat, c.mat, np, save);
    if (h->has_trac && c.tr_fn) {   // they move with the particles at a re-sort
        add(out, h->ps[h->pcur].tr_fn, c.tr_fn, 2 * np, save);
        add(out, h->ps[h->pcur].tr_tau, c.tr_tau, sizeof(float) * 2 * np, save);
    }
    if (h->has_pvc && c.pvc) add(out, h->ps[h->pcur].pvc, c.pvc, 2 * np, save);
    add(out, h->cstart[h->cs_cur], c.cstart, sizeof(int) * ((size_t)h->ncell + 2), save);
    add(out, h->cflag, c.cflag, (size_t)h->ncell, save);
    add(out, h->nvbx, c.nvbx, sizeof(float) * h->nn, save);
    add(out, h->nvby, c.nvby, sizeof(float) * h->nn, save);
    add(out, h->ctl, c.ctl, sizeof(Control), save);
}

void segbuf_free(SegBuf& buf) {
    if (buf.segs) cudaFree(buf.segs);
    if (buf.first) cudaFree(buf.first);
    if (buf.blk) cudaFree(buf.blk);
    buf = SegBuf{};
}

int upload_segments(MpmHandle* h, SegBuf& buf, const std::vector<CopySeg>& segs, cudaStream_t s) {
    buf.nseg = (int)segs.size();
    buf.nblocks = 0;
    if (segs.empty()) return MPM_OK;
    std::vector<unsigned> first(segs.size() + 1);
    unsigned long long total = 0;
    for (size_t i = 0; i < segs.size(); ++i) {
        first[i] = (unsigned)total;
        total += (segs[i].bytes + COPY_CHUNK - 1) / COPY_CHUNK;
    }
    if (total >= 0x7fffffffull) return fail(h, MPM_ERR_INVALID, "state copy too large");
    first[segs.size()] = (unsigned)total;
    if (buf.cap < segs.size() + 1) {
        segbuf_free(buf);
        const size_t cap = segs.size() + 1 + segs.size() / 2;
        CK(h, cudaMalloc(&buf.segs, sizeof(CopySeg) * cap));
        CK(h, cudaMalloc(&buf.first, sizeof(unsigned) * cap));
        buf.cap = cap;
    }
    // (copies from pageable memory return once the host tables are staged)
    CK(h, cudaMemcpyAsync(buf.segs, segs.data(), sizeof(CopySeg) * segs.size(),
                          cudaMemcpyHostToDevice, s));
    CK(h, cudaMemcpyAsync(buf.first, first.data(), sizeof(unsigned) * first.size(),
                          cudaMemcpyHostToDevice, s));
    if (buf.blk_cap < total) {
        if (buf.blk) cudaFree(buf.blk);
        buf.blk = nullptr;
        buf.blk_cap = 0;
        const size_t cap = total + total / 2;
        CK(h, cudaMalloc(&buf.blk, sizeof(CopyChunk) * cap));
        buf.blk_cap = cap;
    }
    CK(h, launch_chunk_table(buf.segs, buf.first, (int)segs.size(), (unsigned)total, buf.blk, s));
    buf.nseg = (int)segs.size();
    buf.nblocks = (unsigned)total;
    return MPM_OK;
}

int run_segments(MpmHandle* h, SegBuf& buf, const std::vector<CopySeg>& segs, cudaStream_t s) {
    TRY(upload_segments(h, buf, segs, s));
    CK(h, launch_copy_segments(buf.blk, buf.nblocks, 0, s));
    return MPM_OK;
}

}  // namespace host
}  // namespace mpm
