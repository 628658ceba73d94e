// One-dimensional explicit MPM on two-node line elements (Linear1D,
// diffmpm/element.py:343-600) -- the same phases as the 2-D step, for meshes
// of `nx` elements of length hx with nodes at float(i) * hx.
//
// Layout: particles are re-sorted by element at the start of every step (the
// 2-D sort machinery with a single row of cells), each element's particles in
// original-index order, and eid[q] holds the element of storage slot q for
// the step.  Node-centric kernels (one thread per node) merge the particles of
// the node's two elements by original index, so every nodal sum adds the
// particle contributions in the order of the reference's sequential scatter
// (a `lax.fori_loop` of `.at[].add`, element.py:138-152): the 1-D step gives
// the oracle's float32 results bit for bit.
//
// Build definitions where the reference's 1-D path does not run as written:
// the element volume is x_{e+1} - x_e (the reference's `ediff1d` broadcast
// only works for one element, element.py:543-546) and the strain rate is
// [dN/dx . v, 0, 0, 0, 0, 0] (the reference indexes a 1 x 1 matrix at [1, 1],
// particle.py:304-305).
#include <cuda_runtime.h>

#include "mpm_device.cuh"
#include "mpm_handle.h"
#include "mpm_kernels.h"

namespace mpm {
namespace {

constexpr int LINE_THREADS = 256;

struct LineElem {
    float x0, x1, c, r;   // nodes, centre, 2 / length
};

__device__ __forceinline__ LineElem line_elem(int e, float h) {
    LineElem g;
    g.x0 = node_coord(e, h);
    g.x1 = node_coord(e + 1, h);
    g.c = fm(fa(g.x0, g.x1), 0.5f);
    g.r = fdv(2.0f, fs(g.x1, g.x0));
    return g;
}

// Shape function of node k (0 left, 1 right) at natural coordinate xi
// (element.py:430-454): (1/2)(1 -/+ xi).
__device__ __forceinline__ float shape2(int k, float xi) {
    return k ? fm(0.5f, fa(1.0f, xi)) : fm(0.5f, fs(1.0f, xi));
}

// dN_k/dx = (-/+ 1/2) * 2 / length (element.py:456-515).
__device__ __forceinline__ float dshape2(int k, float r) { return fm(k ? 0.5f : -0.5f, r); }

// Volume at the per-step reset of solve_jit (particle.py:158-178): element
// length / particles in the element.
__device__ __forceinline__ float reset_volume(const SimDev& S, int e) {
    const LineElem g = line_elem(e, S.hx);
    return fdv(fs(g.x1, g.x0), (float)(S.cstart[e + 1] - S.cstart[e]));
}

// Visit the particles of elements i-1 (as their right node) and i (as their
// left node) in increasing original index; f(q, e, k).
template <class F>
__device__ __forceinline__ void for_node_particles(const SimDev& S, int i, F&& f) {
    int a = 0, ae = 0, b = 0, be = 0;
    if (i >= 1) { a = S.cstart[i - 1]; ae = S.cstart[i]; }
    if (i < S.nx) { b = S.cstart[i]; be = S.cstart[i + 1]; }
    #pragma unroll 1
    while (a < ae || b < be) {
        const bool left = a < ae && (b >= be || S.pid[a] < S.pid[b]);
        if (left) { f(a, i - 1, 1); ++a; }
        else { f(b, i, 0); ++b; }
    }
}

// Nodal constraint of direction 0 (constraint.py:29-44): slot + 1, or 0.
__device__ __forceinline__ int cons0(const SimDev& S, int i) { return S.ncons[i] & 0xff; }

template <bool REINIT>
__global__ void __launch_bounds__(LINE_THREADS)
k_line_nodal_kinematics(const __grid_constant__ SimDev S, int par) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > S.nx) return;
    const float* rho = S.rho[par];
    float m = 0.0f, p = 0.0f;
    for_node_particles(S, i, [&](int q, int e, int k) {
        const LineElem g = line_elem(e, S.hx);
        const float N = shape2(k, natural(S.x[q], g.c, g.r));
        const float mp = REINIT ? fm(reset_volume(S, e), rho[q]) : S.mass[q];
        m = fa(m, fm(mp, N));                       // element.py:138-152
        p = fa(p, fm(N, fm(mp, S.vx[q])));          // element.py:166-184
    });
    p = flush(p);                                    // element.py:185-189
    float v = m == 0.0f ? S.nvbx[i] : fdv(p, m);     // element.py:191-202
    v = flush(v);
    const int c = cons0(S, i);
    if (c) v = S.cons_vel[c - 1];                    // constraint.py:29-44
    S.nm[i] = m;
    S.nvax[i] = v;
    if (c) S.nax[i] = 0.0f;
}

// Strain rate, strain, volume and stress of each particle from the nodal
// velocities `nv` (particle.py:249-327), reading ping-pong slot `par` and
// writing `par ^ 1`.
template <bool REINIT>
__global__ void __launch_bounds__(LINE_THREADS)
k_line_stress(const __grid_constant__ SimDev S, const int* __restrict__ eid,
              const float* __restrict__ nv, int par) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= S.np) return;
    const int e = eid[q];
    const LineElem g = line_elem(e, S.hx);
    const float r = flush(fa(fm(dshape2(0, g.r), nv[e]), fm(dshape2(1, g.r), nv[e + 1])));
    const float dvol = fm(S.dt, r);     // the centroid rate equals r in 1-D
    const int o = par ^ 1;
    PState ps{S.sxx[par][q], S.syy[par][q], S.szz[par][q], S.sxy[par][q],
              S.exx[q], S.eyy[q], S.exy[q], S.rho[par][q], S.vsc[par][q]};
    const MatDev M = S.mats[S.mat[q]];
    const float Ep = S.E ? S.E[q] : -1.0f;
    const float f = strain_stress_update(M, Ep, S.dt, r, 0.0f, 0.0f, dvol, ps);
    S.sxx[o][q] = ps.sxx; S.syy[o][q] = ps.syy; S.szz[o][q] = ps.szz; S.sxy[o][q] = ps.sxy;
    S.exx[q] = ps.exx; S.eyy[q] = ps.eyy; S.exy[q] = ps.exy;
    S.rho[o][q] = ps.rho; S.vsc[o][q] = ps.vsc;
    const float V0 = REINIT ? reset_volume(S, e) : S.vol[par][q];
    S.vol[o][q] = fm(V0, f);            // particle.py:324-327
}

// External and internal nodal forces, then the nodal update
// (element.py:204-329).  `spar` is the slot holding the stress and volume the
// forces use (after the USF update, or before the USL one).
template <bool REINIT>
__global__ void __launch_bounds__(LINE_THREADS)
k_line_forces(const __grid_constant__ SimDev S, int par, int spar, int step) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > S.nx) return;
    const float* rho = S.rho[par];
    const float* sxx = S.sxx[spar];
    const float* vol = S.vol[spar];
    const bool usl_reset = REINIT && spar == par;   // USL under solve_jit: reset volume
    float fext = 0.0f, fint = 0.0f;
    for_node_particles(S, i, [&](int q, int e, int k) {
        const LineElem g = line_elem(e, S.hx);
        const float N = shape2(k, natural(S.x[q], g.c, g.r));
        const float mp = REINIT ? fm(reset_volume(S, e), rho[q]) : S.mass[q];
        fext = fa(fext, fm(N, fm(mp, S.gx)));                       // element.py:236-268
        const float V = usl_reset ? reset_volume(S, e) : vol[q];
        fint = fa(fint, fm(fm(-V, sxx[q]), dshape2(k, g.r)));       // element.py:548-600
    });
    if (S.cnf_ptr) {                                                 // element.py:270-284
        const float t = step_time(step, S.dt);
        #pragma unroll 1
        for (int j = S.cnf_ptr[i]; j < S.cnf_ptr[i + 1]; ++j)
            fext = fa(fext, fm(fn_value(S, S.cnf_fn[j], t), S.cnf_val[j]));
    }
    const float m = S.nm[i];
    float a = nan_to_num(fdv(fa(fa(fint, fext), 0.0f), m));          // element.py:305-329
    float v = fa(S.nvax[i], fm(a, S.dt));
    const int c = cons0(S, i);
    if (c) {
        v = S.cons_vel[c - 1];
        a = 0.0f;
    }
    S.nvbx[i] = flush(v);
    S.nax[i] = flush(a);
}

// G2P (particle.py:208-247) and the element check of the moved particle.
__global__ void __launch_bounds__(LINE_THREADS)
k_line_g2p(const __grid_constant__ SimDev S, const int* __restrict__ eid, Control* __restrict__ ctl) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= S.np) return;
    const int e = eid[q];
    const LineElem g = line_elem(e, S.hx);
    const float xi = natural(S.x[q], g.c, g.r);
    const float N0 = shape2(0, xi), N1 = shape2(1, xi);
    const float vh = fa(fm(N0, S.nvbx[e]), fm(N1, S.nvbx[e + 1]));
    const float ah = fa(fm(N0, S.nax[e]), fm(N1, S.nax[e + 1]));
    float v = S.velocity_update ? vh : fa(S.vx[q], fm(ah, S.dt));
    if (S.pvc && S.pvc[2 * q]) v = S.pvc_vel[S.pvc[2 * q] - 1];   // particle velocity constraint
    S.vx[q] = v;
    const float x = fa(S.x[q], fm(vh, S.dt));
    S.x[q] = x;
    const int ne = locate_axis(x, S.hx, S.nx);
    if (ne < 0 || ne >= S.nx) atomicOr(&ctl->status, ST_OUT_OF_MESH);
}

// Element of each storage slot: the bucket it was sorted into.
__global__ void k_line_eid(const int* __restrict__ cstart, int nx, int* __restrict__ eid) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nx) return;
    #pragma unroll 1
    for (int q = cstart[e]; q < cstart[e + 1]; ++q) eid[q] = e;
}

// Each element's particles in increasing original index (insertion sort of a
// bucket by pid; buckets hold a few particles).
__global__ void k_line_segsort(int nbucket, const int* __restrict__ start, int* __restrict__ perm,
                               const int* __restrict__ pid) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nbucket) return;
    const int b = start[c], e = start[c + 1];
    #pragma unroll 1
    for (int i = b + 1; i < e; ++i) {
        const int v = perm[i];
        const int pv = pid[v];
        int j = i - 1;
        #pragma unroll 1
        while (j >= b && pid[perm[j]] > pv) {
            perm[j + 1] = perm[j];
            --j;
        }
        perm[j + 1] = v;
    }
}

// V = element length / count, m = V rho, size = V (solve semantics set-up,
// particle.py:158-178).
__global__ void k_line_setup_volume(const __grid_constant__ SimDev S, const int* __restrict__ eid, int par) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= S.np) return;
    const float V = reset_volume(S, eid[q]);
    S.vol[par][q] = V;
    S.mass[q] = fm(V, S.rho[par][q]);
    S.psize[q] = V;
}

inline int blocks(int n) { return (n + LINE_THREADS - 1) / LINE_THREADS; }

}  // namespace

cudaError_t launch_line_segsort(int nbucket, const int* start, int* perm, const int* pid, cudaStream_t s) {
    if (nbucket > 0) k_line_segsort<<<blocks(nbucket), LINE_THREADS, 0, s>>>(nbucket, start, perm, pid);
    return cudaGetLastError();
}

cudaError_t launch_line_eid(const int* cstart, int nx, int* eid, cudaStream_t s) {
    if (nx > 0) k_line_eid<<<blocks(nx), LINE_THREADS, 0, s>>>(cstart, nx, eid);
    return cudaGetLastError();
}

namespace host {

int line_setup_volume(MpmHandle* h, cudaStream_t s) {
    if (h->np > 0)
        k_line_setup_volume<<<blocks((int)h->np), LINE_THREADS, 0, s>>>(h->hs, h->line_eid, parity(h));
    CK(h, cudaGetLastError());
    return MPM_OK;
}

// One step: re-sort by element, nodal kinematics, (USF) stress update, forces
// and nodal update, G2P, (USL) stress update.
int line_step(MpmHandle* h, cudaStream_t s, const LineTapeSlot* tape) {
    TRY(resort(h, s));
    const SimDev& S = h->hs;
    const int par = parity(h), nb = blocks(h->nx + 1), pb = blocks((int)h->np);
    const int step = (int)h->step;
    const size_t fb = sizeof(float) * (size_t)h->np, nbytes = sizeof(float) * (size_t)h->nn;
    if (tape) {
        const float* src[9] = {S.x, S.vx, S.sxx[par], S.syy[par], S.szz[par], S.sxy[par], S.rho[par],
                               S.vol[par], S.vsc[par]};
        for (int k = 0; k < 9; ++k) CK(h, cudaMemcpyAsync(tape->p[k], src[k], fb, cudaMemcpyDeviceToDevice, s));
        CK(h, cudaMemcpyAsync(tape->pid, S.pid, sizeof(int) * (size_t)h->np, cudaMemcpyDeviceToDevice, s));
        CK(h, cudaMemcpyAsync(tape->cs, S.cstart, sizeof(int) * (size_t)(h->nx + 2), cudaMemcpyDeviceToDevice, s));
    }
    if (h->reinit) k_line_nodal_kinematics<true><<<nb, LINE_THREADS, 0, s>>>(S, par);
    else k_line_nodal_kinematics<false><<<nb, LINE_THREADS, 0, s>>>(S, par);
    if (!h->usl) {
        if (h->reinit) k_line_stress<true><<<pb, LINE_THREADS, 0, s>>>(S, h->line_eid, h->nvax, par);
        else k_line_stress<false><<<pb, LINE_THREADS, 0, s>>>(S, h->line_eid, h->nvax, par);
    }
    const int spar = h->usl ? par : par ^ 1;
    if (h->reinit) k_line_forces<true><<<nb, LINE_THREADS, 0, s>>>(S, par, spar, step);
    else k_line_forces<false><<<nb, LINE_THREADS, 0, s>>>(S, par, spar, step);
    k_line_g2p<<<pb, LINE_THREADS, 0, s>>>(S, h->line_eid, h->ctl);
    if (h->usl) {
        if (h->reinit) k_line_stress<true><<<pb, LINE_THREADS, 0, s>>>(S, h->line_eid, h->nvbx, par);
        else k_line_stress<false><<<pb, LINE_THREADS, 0, s>>>(S, h->line_eid, h->nvbx, par);
    }
    CK(h, cudaGetLastError());
    if (tape) {
        const float* src[4] = {h->nm, h->nvax, h->nvbx, h->nax};
        for (int k = 0; k < 4; ++k) CK(h, cudaMemcpyAsync(tape->n[k], src[k], nbytes, cudaMemcpyDeviceToDevice, s));
    }
    h->step++;
    h->needs_resort = true;
    return MPM_OK;
}

}  // namespace host
}  // namespace mpm
