// Hand-written adjoint of the 1-D step (mpm_line.cu) under solve_jit
// semantics, USF or USL, LinearElastic (material or per-particle E) and
// SimpleMaterial: the reverse of diffmpm/scheme.py:22-133 on Linear1D
// elements (element.py:343-600), particle.py:208-327.
//
// mpm_record on a 1-D handle keeps a full tape (1-D runs are small): for every
// step its start state in that step's storage order (x, v, the four stress
// components, density, the storage -> original map, the element starts) and
// its nodal results (mass, velocity after kinematics, velocity and acceleration
// after the update).  mpm_adjoint walks the steps backwards; the particle
// adjoints live in original order between steps, so the per-step re-sorts need
// no permutation.  Per step (USL adds pass 0):
//   0 (USL)  particle: reverse of the stress update after G2P (strain-rate
//            adjoint r-bar from the updated nodal velocities);
//   1        particle: reverse of G2P (v-hat bar, a-hat bar; x through N);
//   2        node: transposed G2P (+ USL r-bar), reverse nodal update;
//   3        particle: reverse of the forces (+ USF stress update);
//   4        node: (USF) transposed strain-rate gather, reverse nodal velocity;
//   5        particle: reverse of the mass and momentum sums.
// As in the 2-D adjoint, a component that a flush or a constraint set carries
// no adjoint (masks from the stored values), and the velocity a massless node
// keeps from the previous step is not differentiated.
#include <cuda_runtime.h>

#include <vector>

#include "mpm_device.cuh"
#include "mpm_handle.h"
#include "mpm_kernels.h"

namespace mpm {

enum { LP_X, LP_V, LP_SXX, LP_SYY, LP_SZZ, LP_SXY, LP_RHO, LP_VOL, LP_VSC, LP_N };   // particle tape
enum { LN_M, LN_VA, LN_VB, LN_A, LN_N };                            // nodal tape fields
// particle adjoints (original order)
enum { LA_X, LA_V, LA_SXX, LA_SYY, LA_SZZ, LA_SXY, LA_RHO, LA_VSC, LA_EXX, LA_EYY, LA_EXY, LA_E, LA_VOL,
       LA_N };
// per-step particle scratch (storage order) and nodal scratch
enum { LS_G, LS_H, LS_R, LS_M, LS_X, LS_V, LS_N };
enum { LNS_F, LNS_M, LNS_VA, LNS_P, LNS_N };

struct LineAdjoint {
    int T = 0;                 // recorded steps
    int64_t np = 0, nn = 0;
    int nx = 0;
    uint64_t gen = 0;
    bool valid = false;
    float* P = nullptr;        // [T][LP_N][np]
    int* pid = nullptr;        // [T][np]
    int* cs = nullptr;         // [T][nx + 2]
    float* N = nullptr;        // [T][LN_N][nn]
    uint8_t* mat0 = nullptr;   // material ids, original order
    uint8_t* pvc0 = nullptr;   // velocity constraint codes, original order (or null)
    float* mass0 = nullptr;    // solve semantics: the constant particle mass, original order
    float* E0 = nullptr;       // per-particle Young's modulus, original order (or null)
    int* eid = nullptr;        // element of each storage slot of the step being reversed
    float* L = nullptr;        // [LA_N][np]
    float* sc = nullptr;       // [LS_N][np]
    float* ns = nullptr;       // [LNS_N][nn]
    std::vector<void*> allocs;
};

namespace {

constexpr int LA_THREADS = 256;
inline int lblocks(int64_t n) { return (int)((n + LA_THREADS - 1) / LA_THREADS); }

// Arguments of one reversed step.
struct LineStep {
    int np, nx, usl, velocity_update, reinit;
    float hx, dt, gx;
    const float* x; const float* v; const float* sxx; const float* syy; const float* szz;
    const float* sxy; const float* rho; const float* vol; const float* vsc;
    const int* pid; const int* cs; const int* eid;
    const float* M; const float* vA; const float* vB; const float* a;
    const uint16_t* ncons;
    const MatDev* mats; const uint8_t* mat0; const float* E0;
    const uint8_t* pvc0;
    const float* mass0;
    float* L[LA_N];
    float* sc[LS_N];
    float* ns[LNS_N];
};

struct Elem {
    float c, r, V0;   // centre, 2 / length, reset volume
};

__device__ __forceinline__ Elem elem_of(const LineStep& A, int e) {
    const float x0 = node_coord(e, A.hx), x1 = node_coord(e + 1, A.hx);
    Elem g;
    g.c = fm(fa(x0, x1), 0.5f);
    g.r = fdv(2.0f, fs(x1, x0));
    g.V0 = fdv(fs(x1, x0), (float)(A.cs[e + 1] - A.cs[e]));
    return g;
}

__device__ __forceinline__ void shapes(const Elem& g, float x, float& N0, float& N1, float& d0,
                                       float& d1) {
    const float xi = natural(x, g.c, g.r);
    N0 = fm(0.5f, fs(1.0f, xi));
    N1 = fm(0.5f, fa(1.0f, xi));
    d0 = fm(-0.5f, g.r);
    d1 = fm(0.5f, g.r);
}

// Visit the particles of elements i-1 (right node) and i (left node) of the
// step in increasing original index: f(q, e, k).
template <class F>
__device__ __forceinline__ void for_node(const LineStep& A, int i, F&& f) {
    int a = 0, ae = 0, b = 0, be = 0;
    if (i >= 1) { a = A.cs[i - 1]; ae = A.cs[i]; }
    if (i < A.nx) { b = A.cs[i]; be = A.cs[i + 1]; }
    #pragma unroll 1
    while (a < ae || b < be) {
        const bool left = a < ae && (b >= be || A.pid[a] < A.pid[b]);
        if (left) { f(a, i - 1, 1); ++a; }
        else { f(b, i, 0); ++b; }
    }
}

// Reverse of the strain / volume / density / stress update driven by the
// nodal velocities nv (particle.py:249-327, material.py:113-131 and the
// build's Newtonian total stress) at slot q: given the adjoints of the updated
// stress (sb, by component; xx may carry the forces' share), density,
// centroid strain and strain, of the updated volume used by the USF forces
// (Vb) and, under solve semantics, carried to the next step (L[LA_VOL]),
// returns r-bar (zero when the rate was flushed), adds dL/dE and writes the
// start-of-step adjoints.  V0 is the volume the update starts from.
__device__ __forceinline__ float rev_stress(const LineStep& A, int q, int o, int e, float V0,
                                            const float* nv, const float sb[4], float Vb) {
    const Elem g = elem_of(A, e);
    const float d0n = fm(-0.5f, g.r), d1n = fm(0.5f, g.r);
    const float raw = fa(fm(d0n, nv[e]), fm(d1n, nv[e + 1]));
    const float r = flush(raw);
    const float dvol = fm(A.dt, r), f = fa(1.0f, dvol), d0 = fm(r, A.dt);
    const MatDev M = A.mats[A.mat0[o]];
    const float Ep = A.E0 ? A.E0[o] : -1.0f;
    float rb = 0.0f, Eb = 0.0f, vscb = 0.0f;
    bool total = false;
    if (M.type == MAT_LINEAR_ELASTIC) {
        float a1 = M.a1, a2 = M.a2;
        if (Ep >= 0.0f) {
            a1 = fm(Ep, M.c1);
            a2 = fm(Ep, M.c2);
        }
        rb = fm(A.dt, fa(fa(fm(a1, sb[0]), fm(a2, sb[1])), fm(a2, sb[2])));
        Eb = fm(d0, fa(fa(fm(M.c1, sb[0]), fm(M.c2, sb[1])), fm(M.c2, sb[2])));
    } else if (M.type == MAT_SIMPLE) {   // sigma += E * deps (only the xx strain moves in 1-D)
        rb = fm(A.dt, fm(Ep >= 0.0f ? Ep : M.E, sb[0]));
        Eb = fm(d0, sb[0]);
    } else {   // Newtonian: sigma = K vsc' I + 2 mu dev(r), r = (r, 0, 0)
        const float tr = fa(fa(sb[0], sb[1]), sb[2]);
        rb = fa(fm(M.twomu, sb[0]), fdv(-fm(M.twomu, tr), 3.0f));
        vscb = fm(M.K, tr);
        total = true;
    }
    const float rho0 = A.rho[q];
    const float rhob1 = A.L[LA_RHO][o];
    // rho' = rho / f, V = V0 f, vsc' = vsc + dvol, exx' = exx + r dt
    const float Vt = A.reinit ? Vb : fa(Vb, A.L[LA_VOL][o]);
    float fb = fm(V0, Vt);
    fb = fs(fb, fdv(fm(rhob1, fdv(rho0, f)), f));
    const float vscb1 = fa(A.L[LA_VSC][o], vscb);
    const float dvolb = fa(fb, vscb1);
    rb = fa(rb, fm(A.dt, fa(dvolb, A.L[LA_EXX][o])));
    if (r == 0.0f) rb = 0.0f;
    A.L[LA_RHO][o] = fdv(rhob1, f);
    A.L[LA_VSC][o] = vscb1;
    if (!A.reinit) A.L[LA_VOL][o] = fm(Vt, f);
    A.L[LA_SXX][o] = total ? 0.0f : sb[0];
    A.L[LA_SYY][o] = total ? 0.0f : sb[1];
    A.L[LA_SZZ][o] = total ? 0.0f : sb[2];
    A.L[LA_SXY][o] = total ? 0.0f : sb[3];
    A.L[LA_E][o] = fa(A.L[LA_E][o], Eb);
    return rb;
}

// The volume a step's stress update starts from: the per-step set-up
// (element length / count) or, under solve semantics, the carried volume.
__device__ __forceinline__ float start_volume(const LineStep& A, int q, int e) {
    return A.reinit ? elem_of(A, e).V0 : A.vol[q];
}

// pass 0 (USL): the stress update after G2P used the updated velocities
__global__ void k_lrev0(const __grid_constant__ LineStep A) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= A.np) return;
    const int o = A.pid[q], e = A.eid[q];
    const float sb[4] = {A.L[LA_SXX][o], A.L[LA_SYY][o], A.L[LA_SZZ][o], A.L[LA_SXY][o]};
    A.sc[LS_R][q] = rev_stress(A, q, o, e, start_volume(A, q, e), A.vB, sb, 0.0f);
}

// pass 1: G2P (particle.py:208-247)
__global__ void k_lrev1(const __grid_constant__ LineStep A) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= A.np) return;
    const int o = A.pid[q], e = A.eid[q];
    const Elem g = elem_of(A, e);
    float N0, N1, d0, d1;
    shapes(g, A.x[q], N0, N1, d0, d1);
    // a constrained end velocity (particle velocity constraint) is a constant
    const float lx = A.L[LA_X][o], lv = (A.pvc0 && A.pvc0[o]) ? 0.0f : A.L[LA_V][o];
    const float gh = fa(fm(lx, A.dt), A.velocity_update ? lv : 0.0f);
    const float hh = A.velocity_update ? 0.0f : fm(lv, A.dt);
    A.sc[LS_G][q] = gh;
    A.sc[LS_H][q] = hh;
    const float dv = fa(fm(d0, A.vB[e]), fm(d1, A.vB[e + 1]));
    const float da = fa(fm(d0, A.a[e]), fm(d1, A.a[e + 1]));
    A.sc[LS_X][q] = fa(lx, fa(fm(gh, dv), fm(hh, da)));
    A.sc[LS_V][q] = A.velocity_update ? 0.0f : lv;
}

// pass 2: transposed G2P (and USL strain-rate gather), reverse nodal update
// (element.py:305-329)
__global__ void k_lrev2(const __grid_constant__ LineStep A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > A.nx) return;
    float vbb = 0.0f, ab = 0.0f;
    for_node(A, i, [&](int q, int e, int k) {
        const Elem g = elem_of(A, e);
        float N0, N1, d0, d1;
        shapes(g, A.x[q], N0, N1, d0, d1);
        const float N = k ? N1 : N0;
        vbb = fa(vbb, fm(N, A.sc[LS_G][q]));
        ab = fa(ab, fm(N, A.sc[LS_H][q]));
        if (A.usl) vbb = fa(vbb, fm(k ? d1 : d0, A.sc[LS_R][q]));
    });
    const bool cons = (A.ncons[i] & 0xff) != 0;
    if (cons || A.vB[i] == 0.0f) vbb = 0.0f;
    if (cons || A.a[i] == 0.0f) ab = 0.0f;
    const float at = fa(ab, fm(vbb, A.dt));
    const float M = A.M[i];
    float Fb = 0.0f, Mb = 0.0f;
    if (M != 0.0f && at != 0.0f) {
        Fb = fdv(at, M);
        Mb = -fdv(fm(at, A.a[i]), M);
    }
    A.ns[LNS_F][i] = Fb;
    A.ns[LNS_M][i] = Mb;
    A.ns[LNS_VA][i] = vbb;
}

// pass 3: forces (element.py:236-268, 548-600) and the USF stress update
template <bool USL>
__global__ void k_lrev3(const __grid_constant__ LineStep A) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= A.np) return;
    const int o = A.pid[q], e = A.eid[q];
    const Elem g = elem_of(A, e);
    float N0, N1, d0, d1;
    shapes(g, A.x[q], N0, N1, d0, d1);
    const float F0 = A.ns[LNS_F][e], F1 = A.ns[LNS_F][e + 1];
    const float SF = fa(fm(N0, F0), fm(N1, F1)), SD = fa(fm(d0, F0), fm(d1, F1));
    const float V0 = start_volume(A, q, e);
    const float m = A.reinit ? fm(g.V0, A.rho[q]) : A.mass0[o];
    float xb = fa(A.sc[LS_X][q], fm(fm(m, A.gx), SD));
    float mb = fm(A.gx, SF);
    // the stress and volume the forces used (USF: after this step's update)
    float sxx = A.sxx[q], V = V0;
    if (!USL) {
        const float r = flush(fa(fm(fm(-0.5f, g.r), A.vA[e]), fm(fm(0.5f, g.r), A.vA[e + 1])));
        PState ps{A.sxx[q], A.syy[q], A.szz[q], A.sxy[q], 0.0f, 0.0f, 0.0f, A.rho[q], A.vsc[q]};
        const float f = strain_stress_update(A.mats[A.mat0[o]], A.E0 ? A.E0[o] : -1.0f, A.dt, r,
                                             0.0f, 0.0f, fm(A.dt, r), ps);
        sxx = ps.sxx;
        V = fm(V0, f);
    }
    const float sxxb = fm(-V, SD);   // d F_i / d sxx = -V dN_i
    const float Vb = fm(-sxx, SD);
    if (USL) {
        A.L[LA_SXX][o] = fa(A.L[LA_SXX][o], sxxb);
        if (!A.reinit) A.L[LA_VOL][o] = fa(A.L[LA_VOL][o], Vb);   // the start volume
        A.sc[LS_R][q] = 0.0f;
    } else {
        const float sb[4] = {fa(A.L[LA_SXX][o], sxxb), A.L[LA_SYY][o], A.L[LA_SZZ][o], A.L[LA_SXY][o]};
        A.sc[LS_R][q] = rev_stress(A, q, o, e, V0, A.vA, sb, Vb);
    }
    A.sc[LS_X][q] = xb;
    A.sc[LS_M][q] = mb;
}

// pass 4: (USF) transposed strain-rate gather, reverse nodal velocity
// (element.py:191-202, 331-334)
__global__ void k_lrev4(const __grid_constant__ LineStep A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > A.nx) return;
    float vab = A.ns[LNS_VA][i];
    if (!A.usl) {
        for_node(A, i, [&](int q, int e, int k) {
            const Elem g = elem_of(A, e);
            vab = fa(vab, fm(fm(k ? 0.5f : -0.5f, g.r), A.sc[LS_R][q]));
        });
    }
    const bool cons = (A.ncons[i] & 0xff) != 0;
    const float M = A.M[i], va = A.vA[i];
    float Pb = 0.0f, Mb = A.ns[LNS_M][i];
    if (!cons && M != 0.0f && va != 0.0f) {
        Pb = fdv(vab, M);
        Mb = fs(Mb, fdv(fm(vab, va), M));
    }
    A.ns[LNS_P][i] = Pb;
    A.ns[LNS_M][i] = Mb;
}

// pass 5: mass and momentum (element.py:122-189) and m = V0 rho
__global__ void k_lrev5(const __grid_constant__ LineStep A) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= A.np) return;
    const int o = A.pid[q], e = A.eid[q];
    const Elem g = elem_of(A, e);
    float N0, N1, d0, d1;
    shapes(g, A.x[q], N0, N1, d0, d1);
    const float M0 = A.ns[LNS_M][e], M1 = A.ns[LNS_M][e + 1];
    const float P0 = A.ns[LNS_P][e], P1 = A.ns[LNS_P][e + 1];
    const float m = A.reinit ? fm(g.V0, A.rho[q]) : A.mass0[o], v = A.v[q];
    const float SM = fa(fm(N0, M0), fm(N1, M1)), SP = fa(fm(N0, P0), fm(N1, P1));
    const float DM = fa(fm(d0, M0), fm(d1, M1)), DP = fa(fm(d0, P0), fm(d1, P1));
    const float mb = fa(A.sc[LS_M][q], fa(SM, fm(v, SP)));
    A.L[LA_X][o] = fa(A.sc[LS_X][q], fa(fm(m, DM), fm(fm(m, v), DP)));
    A.L[LA_V][o] = fa(A.sc[LS_V][q], fm(m, SP));
    if (A.reinit) A.L[LA_RHO][o] = fa(A.L[LA_RHO][o], fm(g.V0, mb));   // m = V0 rho
}

// A float per particle from storage to original order.
__global__ void k_lscatter(const float* __restrict__ src, const int* __restrict__ pid, int np,
                           float* __restrict__ out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < np) out[pid[q]] = src[q];
}

// Material ids (or every `stride`-th byte of a per-particle code array) from
// storage to original order.
__global__ void k_lmat0(const uint8_t* __restrict__ mat, const int* __restrict__ pid, int np,
                        int stride, uint8_t* __restrict__ out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < np) out[pid[q]] = mat[(size_t)q * stride];
}

__global__ void k_lfill(float* __restrict__ p, int64_t n, float v) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

}  // namespace

namespace host {
namespace {

template <class T>
int line_alloc(MpmHandle* h, LineAdjoint* a, T** p, size_t n) {
    cudaError_t e = cudaMalloc(p, sizeof(T) * (n ? n : 1));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(h, MPM_ERR_NOMEM, "recording: cudaMalloc of %zu bytes failed", sizeof(T) * n);
    }
    a->allocs.push_back(*p);
    return MPM_OK;
}



}  // namespace
}  // namespace host

void line_adjoint_free(MpmHandle* h) {
    if (!h->line_adj) return;
    for (void* p : h->line_adj->allocs) cudaFree(p);
    delete h->line_adj;
    h->line_adj = nullptr;
}

int line_record(MpmHandle* h, int nsteps, cudaStream_t s) {
    using namespace host;
    if (!h->initialized) return fail(h, MPM_ERR_STATE, "initialize first");
    if (nsteps < 1) return fail(h, MPM_ERR_INVALID, "nsteps must be >= 1");
    if (h->np <= 0) return fail(h, MPM_ERR_STATE, "no particles");
    line_adjoint_free(h);
    LineAdjoint* a = new LineAdjoint();
    h->line_adj = a;
    a->T = nsteps;
    a->np = h->np;
    a->nn = h->nn;
    a->nx = h->nx;
    const size_t np = (size_t)h->np, nn = (size_t)h->nn, T = (size_t)nsteps;
    const size_t bytes = T * (np * (LP_N + 1) + (size_t)(h->nx + 2) + nn * LN_N) * 4;
    if (bytes > ((size_t)64 << 30))
        return fail(h, MPM_ERR_NOMEM, "a 1-D recording of %d steps needs %zu bytes", nsteps, bytes);
    TRY(line_alloc(h, a, &a->P, T * LP_N * np));
    TRY(line_alloc(h, a, &a->pid, T * np));
    TRY(line_alloc(h, a, &a->cs, T * (size_t)(h->nx + 2)));
    TRY(line_alloc(h, a, &a->N, T * LN_N * nn));
    TRY(line_alloc(h, a, &a->mat0, np));
    TRY(line_alloc(h, a, &a->eid, np));
    TRY(line_alloc(h, a, &a->L, (size_t)LA_N * np));
    TRY(line_alloc(h, a, &a->sc, (size_t)LS_N * np));
    TRY(line_alloc(h, a, &a->ns, (size_t)LNS_N * nn));
    const PSet& p = h->ps[h->pcur];
    if (np > 0) k_lmat0<<<lblocks((int64_t)np), LA_THREADS, 0, s>>>(p.mat, p.pid, (int)np, 1, a->mat0);
    if (!h->reinit) {   // solve semantics: the constant mass
        TRY(line_alloc(h, a, &a->mass0, np));
        if (np > 0) k_lscatter<<<lblocks((int64_t)np), LA_THREADS, 0, s>>>(p.mass, p.pid, (int)np, a->mass0);
    }
    if (h->has_pvc) {
        TRY(line_alloc(h, a, &a->pvc0, np));
        if (np > 0) k_lmat0<<<lblocks((int64_t)np), LA_THREADS, 0, s>>>(p.pvc, p.pid, (int)np, 2, a->pvc0);
    }
    CK(h, cudaGetLastError());
    if (h->has_E) {
        TRY(line_alloc(h, a, &a->E0, np));
        TRY(gather_field(h, MPM_FIELD_YOUNGS_MODULUS, a->E0, s));
    }
    for (int t = 0; t < nsteps; ++t) {
        LineTapeSlot slot;
        for (int k = 0; k < LP_N; ++k) slot.p[k] = a->P + ((size_t)t * LP_N + k) * np;
        slot.pid = a->pid + (size_t)t * np;
        slot.cs = a->cs + (size_t)t * (h->nx + 2);
        for (int k = 0; k < LN_N; ++k) slot.n[k] = a->N + ((size_t)t * LN_N + k) * nn;
        TRY(line_step(h, s, &slot));
    }
    TRY(read_ctl(h, s));
    int st = h->h_ctl->status;
    TRY(check_status(h, st));
    TRY(clear_status(h, s));
    TRY(sync(h, s));
    h->gen++;
    a->gen = h->gen;
    a->valid = true;
    return MPM_OK;
}

int line_adjoint(MpmHandle* h, const float* dl_dloc, const float* dl_dvel, float* dl_dE,
                 float* dl_dloc0, float* dl_dvel0, int on_device, cudaStream_t s) {
    using namespace host;
    LineAdjoint* a = h->line_adj;
    if (!a || !a->valid || a->gen != h->gen)
        return fail(h, MPM_ERR_STATE, "record the run (mpm_record) right before its adjoint");
    if (!dl_dloc) return fail(h, MPM_ERR_INVALID, "dl_dloc is null");
    const int64_t np = a->np;
    const size_t fb = sizeof(float) * (size_t)np;
    float* L = a->L;
    const int fill_blocks = lblocks((int64_t)LA_N * np);
    k_lfill<<<fill_blocks, LA_THREADS, 0, s>>>(L, (int64_t)LA_N * np, 0.0f);
    const cudaMemcpyKind in = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    CK(h, cudaMemcpyAsync(L + (size_t)LA_X * np, dl_dloc, fb, in, s));
    if (dl_dvel) CK(h, cudaMemcpyAsync(L + (size_t)LA_V * np, dl_dvel, fb, in, s));
    LineStep A{};
    A.np = (int)np;
    A.nx = a->nx;
    A.usl = h->usl ? 1 : 0;
    A.velocity_update = h->velocity_update;
    A.reinit = h->reinit ? 1 : 0;
    A.mass0 = a->mass0;
    A.hx = h->hx;
    A.dt = h->dt;
    A.gx = h->gx;
    A.eid = a->eid;
    A.ncons = h->d_ncons;
    A.mats = h->d_mats;
    A.mat0 = a->mat0;
    A.E0 = a->E0;
    A.pvc0 = a->pvc0;
    for (int k = 0; k < LA_N; ++k) A.L[k] = L + (size_t)k * np;
    for (int k = 0; k < LS_N; ++k) A.sc[k] = a->sc + (size_t)k * np;
    for (int k = 0; k < LNS_N; ++k) A.ns[k] = a->ns + (size_t)k * a->nn;
    const int pb = lblocks(np), nb = lblocks(a->nx + 1);
    for (int t = a->T - 1; t >= 0; --t) {
        const float* P = a->P + (size_t)t * LP_N * np;
        A.x = P + LP_X * np; A.v = P + LP_V * np;
        A.sxx = P + LP_SXX * np; A.syy = P + LP_SYY * np; A.szz = P + LP_SZZ * np;
        A.sxy = P + LP_SXY * np; A.rho = P + LP_RHO * np;
        A.vol = P + LP_VOL * np; A.vsc = P + LP_VSC * np;
        A.pid = a->pid + (size_t)t * np;
        A.cs = a->cs + (size_t)t * (a->nx + 2);
        const float* N = a->N + (size_t)t * LN_N * a->nn;
        A.M = N + LN_M * a->nn; A.vA = N + LN_VA * a->nn;
        A.vB = N + LN_VB * a->nn; A.a = N + LN_A * a->nn;
        CK(h, launch_line_eid(A.cs, a->nx, a->eid, s));
        if (A.usl) k_lrev0<<<pb, LA_THREADS, 0, s>>>(A);
        k_lrev1<<<pb, LA_THREADS, 0, s>>>(A);
        k_lrev2<<<nb, LA_THREADS, 0, s>>>(A);
        if (A.usl) k_lrev3<true><<<pb, LA_THREADS, 0, s>>>(A);
        else k_lrev3<false><<<pb, LA_THREADS, 0, s>>>(A);
        k_lrev4<<<nb, LA_THREADS, 0, s>>>(A);
        k_lrev5<<<pb, LA_THREADS, 0, s>>>(A);
        CK(h, cudaGetLastError());
    }
    const cudaMemcpyKind out = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (dl_dE) CK(h, cudaMemcpyAsync(dl_dE, L + (size_t)LA_E * np, fb, out, s));
    if (dl_dloc0) CK(h, cudaMemcpyAsync(dl_dloc0, L + (size_t)LA_X * np, fb, out, s));
    if (dl_dvel0) CK(h, cudaMemcpyAsync(dl_dvel0, L + (size_t)LA_V * np, fb, out, s));
    return sync(h, s);
}

}  // namespace mpm
