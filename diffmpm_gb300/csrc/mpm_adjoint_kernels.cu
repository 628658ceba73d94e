// Reverse passes of the explicit MPM step (USF or USL, per-step volume set-up).
//
// Notation of the forward USF step, particle p in cell c with corners k = 0..3
// (diffmpm/element.py, particle.py; the step order of diffmpm/scheme.py:22-67;
// USL, scheme.py:112-133, uses sig and V0 in F and updates sig, rho after G2P
// with r = flush(G^T vB), c = flush(Gc^T vB) at the start-of-step positions):
//   m    = V0 rho,           V0 = V_el / count(c)            (solver.py:81-85)
//   M_n  = sum N m,  P_n = flush(sum N m v),  vA = C(flush(P / M))
//   r    = flush(G^T vA) (xx, yy, xy),  c = flush(Gc^T vA),  dvol = dt (c0 + c1)
//   sig' = sig + D(E) r dt,  V = V0 (1 + dvol),  rho' = rho / (1 + dvol)
//   F_n  = sum -V (Gx sxx' + Gy sxy', Gy syy' + Gx sxy') + N m g
//   a    = F / M,  vB = flush(C(vA + a dt)),  aB = flush(C0(a))
//   v'   = velocity_update ? sum N vB : v + dt sum N aB,  x' = x + dt sum N vB
// C sets constrained velocity components, C0 zeroes constrained accelerations.
// flush(a) = 0 for |a| < 1e-12, so its derivative is 0 there and 1 elsewhere:
// a component that is exactly 0 after the flush passes no adjoint.  Cell ids,
// counts and masks are piecewise constant in the positions and pass none.
// The velocity a node with zero mass keeps from the previous step only
// reaches particles whose shape function at that node is exactly zero, so its
// dependence is dropped.
#include <cuda_runtime.h>
#include <cstdint>
#include "mpm_adjoint.h"
#include "mpm_device.cuh"

namespace mpm {

namespace {

constexpr int PART_THREADS = 256;
static_assert(PART_THREADS == ADJ_BLOCK, "the batched block map counts ADJ_BLOCK particles per chunk");

// Particles currently in cell (ci, cj) at the step start, in the order of the
// forward gathers: the cell's own sort-cell, and neighbouring sort-cells whose
// drift flag is set (positions tested).
template <class F>
__device__ __forceinline__ void visit_tape_cell(const AdjStep& A, int ci, int cj, const CellGeo& g,
                                                F&& f) {
    #pragma unroll 1
    for (int dj = -1; dj <= 1; ++dj) {
        const int sj = cj + dj;
        if (sj < 0 || sj >= A.ny) continue;
        #pragma unroll 1
        for (int di = -1; di <= 1; ++di) {
            const int si = ci + di;
            if (si < 0 || si >= A.nx) continue;
            const int s = sj * A.nx + si;
            const bool flagged = A.cflag[s] != 0;
            if (!(di == 0 && dj == 0) && !flagged) continue;
            const int b = A.cstart[s], e = A.cstart[s + 1];
            #pragma unroll 1
            for (int q = b; q < e; ++q) {
                if (flagged && !in_cell(g, A.x[q], A.y[q])) continue;
                f(q);
            }
        }
    }
}

__device__ __forceinline__ void particle_cell(const AdjStep& A, float x, float y, int& ci, int& cj) {
    ci = min(max(locate_axis(x, A.hx, A.nx), 0), A.nx - 1);
    cj = min(max(locate_axis(y, A.hy, A.ny), 0), A.ny - 1);
}

// Batched launches: the CTA copies its simulation's arguments into shared
// memory (one word per thread).
__device__ __forceinline__ void load_step_args(const AdjStep* __restrict__ src, AdjStep& dst) {
    static_assert(sizeof(AdjStep) % 4 == 0, "arguments copied in 4-byte words");
    const int* a = reinterpret_cast<const int*>(src);
    int* b = reinterpret_cast<int*>(&dst);
    for (int i = threadIdx.x; i < (int)(sizeof(AdjStep) / 4); i += blockDim.x) b[i] = a[i];
    __syncthreads();
}

// Adjoint seeds of G2P: (v-hat bar, a-hat bar) of particle q.
__device__ __forceinline__ void g2p_seeds(const AdjStep& A, int q, float& gx, float& gy,
                                          float& hx, float& hy) {
    const float lvx = A.lvx[q], lvy = A.lvy[q];
    gx = fm(A.lx[q], A.dt);
    gy = fm(A.ly[q], A.dt);
    if (A.velocity_update) {
        gx = fa(gx, lvx);
        gy = fa(gy, lvy);
        hx = 0.0f;
        hy = 0.0f;
    } else {
        hx = fm(lvx, A.dt);
        hy = fm(lvy, A.dt);
    }
}

// ---------------------------------------------------------------------------
// Tiles of the two node passes: the forward kernels' tiles (a CTA of
// TILE_THREADS threads covers TILE_CX x TILE_CY cells and owns the nodes at
// the upper-right corners of all but its first column and row), with each
// thread summing the corner contributions of its cell's particles.  Fast
// path: the cell rows are staged with coalesced 16-byte copies (row_pass16); slow path
// (a particle near the tile was outside its sort-cell at the step start): the
// tape's drift flags and visit_tape_cell.  Tiles with no stored particle in
// reach only write their nodes (all sums zero).
// ---------------------------------------------------------------------------

// Slots of a staged row per pass of the reverse node passes: a row of 4
// particles in each of 32 cells, starting anywhere in a 16-byte piece, fits
// one pass.  The staged arrays (tape slots, adjoint and scratch arrays) start
// on 16-byte boundaries and hold a multiple of 4 slots.
constexpr int REV_ROW_P = 132;

// Tile set-up of the reverse node passes with every load issued before any is
// consumed (one round trip): this thread's storage start of row cj (cs, and
// cs32 for lane 0), and its shares of two block-wide ORs: a particle is stored
// in the sort-cells around the tile (occ), one of them has a drift flag (drift).
__device__ __forceinline__ void rev_tile_loads(const AdjStep& A, int c0x, int c0y, int cj, int lane,
                                               int& cs, int& cs32, int& occ, int& drift) {
    cs = cs32 = occ = drift = 0;
    if (cj >= 0 && cj < A.ny) {
        const int base = cj * A.nx;
        cs = A.cstart[base + min(max(c0x + lane, 0), A.nx)];
        if (lane == 0) cs32 = A.cstart[base + min(max(c0x + 32, 0), A.nx)];
    }
    const int x0 = max(c0x - 1, 0), x1 = min(c0x + TILE_CX + 1, A.nx);
    const int y0 = max(c0y - 1, 0), y1 = min(c0y + TILE_CY + 1, A.ny);
    if (x0 < x1)
        for (int r = y0 + (int)threadIdx.x; r < y1; r += blockDim.x)
            occ |= A.cstart[r * A.nx + x1] != A.cstart[r * A.nx + x0];
    for (int idx = threadIdx.x; idx < (TILE_CX + 2) * (TILE_CY + 2); idx += blockDim.x) {
        const int si = c0x - 1 + idx % (TILE_CX + 2), sj = c0y - 1 + idx / (TILE_CX + 2);
        if (si >= 0 && si < A.nx && sj >= 0 && sj < A.ny) drift |= A.cflag[sj * A.nx + si];
    }
}

// Reverse nodal update of node n from the G2P adjoint sums (vB-bar, aB-bar):
// vB = flush(C(vA + a dt)), aB = flush(C0(a)), a = F / M (element.py:305-329).
// USL adds the vB-bar of its stress update, gathered by pass G into vabx, vaby.
template <bool USL>
__device__ __forceinline__ void rev_node_update(const AdjStep& A, int n, float vbx, float vby,
                                                float abx, float aby) {
    if (USL) {
        vbx = fa(vbx, A.vabx[n]);
        vby = fa(vby, A.vaby[n]);
    }
    float fbx = 0.0f, fby = 0.0f, mb = 0.0f, wbx = 0.0f, wby = 0.0f;
    const float M = A.nm[n];
    if (M != 0.0f) {
        const uint16_t code = A.ncons[n];
        const bool cx = (code & 0xff) != 0, cy = (code >> 8) != 0;
        const float vBx = A.nvbx[n], vBy = A.nvby[n], aBx = A.nax[n], aBy = A.nay[n];
        wbx = (cx || vBx == 0.0f) ? 0.0f : vbx;
        wby = (cy || vBy == 0.0f) ? 0.0f : vby;
        const float ax = fa((cx || aBx == 0.0f) ? 0.0f : abx, fm(wbx, A.dt));
        const float ay = fa((cy || aBy == 0.0f) ? 0.0f : aby, fm(wby, A.dt));
        fbx = fdv(ax, M);
        fby = fdv(ay, M);
        mb = -fdv(fa(fm(ax, aBx), fm(ay, aBy)), M);
    }
    A.fbx[n] = fbx;
    A.fby[n] = fby;
    A.mb[n] = mb;
    A.vabx[n] = wbx;
    A.vaby[n] = wby;
}

// ---------------------------------------------------------------------------
// Pass 1: transposed G2P (v-hat bar = x-bar dt [+ v-bar], a-hat bar = v-bar dt
// gathered to the nodes with the shape functions), the reverse nodal update
// and the particle count of every cell (particle.py:208-247, element.py:305-329).
// ---------------------------------------------------------------------------
template <bool USL>
__device__ __forceinline__ void rev_nodal_update_tile(const AdjStep& A, const int4 T) {
    constexpr int NQ = 16;   // [v-hat bar x, y, a-hat bar x, y] x corner
    __shared__ float s_c[NQ][SC_STRIDE];
    __shared__ __align__(16) float s_row[TILE_CY][6][REV_ROW_P];
    __shared__ int s_cs[TILE_CY][33];
    const int tid = threadIdx.x, tx = tid % TILE_CX, ty = tid / TILE_CX;
    const int c0x = T.y * TILE_NX - 1, c0y = T.z * TILE_NY - 1;
    const int ci = c0x + tx, cj = c0y + ty;
    const bool node_ok = tx < TILE_NX && ty < TILE_NY && c0x + 1 + tx <= A.nx && c0y + 1 + ty <= A.ny;
    const int node = (c0y + 1 + ty) * (A.nx + 1) + c0x + 1 + tx;
    const bool own_cell = tx >= 1 && ty >= 1 && ci < A.nx && cj < A.ny;
    float sum[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    int L_cs, L_cs32, L_occ, L_drift;
    rev_tile_loads(A, c0x, c0y, cj, tx, L_cs, L_cs32, L_occ, L_drift);
    s_cs[ty][tx] = L_cs;
    if (tx == 0) s_cs[ty][32] = L_cs32;
    if (__syncthreads_or(L_occ)) {
        const bool slow = __syncthreads_or(L_drift) != 0;
        const bool in_mesh = ci >= 0 && ci < A.nx && cj >= 0 && cj < A.ny;
        const CellGeo g = cell_geo(ci, cj, A.hx, A.hy);
        float acc[NQ];
        #pragma unroll
        for (int k = 0; k < NQ; ++k) acc[k] = 0.0f;
        int cnt = 0;
        auto add = [&](float x, float y, float lxv, float lyv, float lvx, float lvy) {
            float N[4];
            shape4(natural(x, g.cx, g.rx), natural(y, g.cy, g.ry), N);
            float gx = fm(lxv, A.dt), gy = fm(lyv, A.dt), hx = 0.0f, hy = 0.0f;
            if (A.velocity_update) {
                gx = fa(gx, lvx);
                gy = fa(gy, lvy);
            } else {
                hx = fm(lvx, A.dt);
                hy = fm(lvy, A.dt);
            }
            #pragma unroll
            for (int k = 0; k < 4; ++k) {
                acc[k] = fa(acc[k], fm(N[k], gx));
                acc[4 + k] = fa(acc[4 + k], fm(N[k], gy));
                acc[8 + k] = fa(acc[8 + k], fm(N[k], hx));
                acc[12 + k] = fa(acc[12 + k], fm(N[k], hy));
            }
            ++cnt;
        };
        if (!slow) {
            const int* cs = s_cs[ty];
            const float* const src[6] = {A.x, A.y, A.lx, A.ly, A.lvx, A.lvy};
            float (*buf)[REV_ROW_P] = s_row[ty];
            row_pass16<6, REV_ROW_P>(buf, src, cs[0], cs[32], cs[tx], cs[tx + 1], tx, [&](int, int j) {
                add(buf[0][j], buf[1][j], buf[2][j], buf[3][j], buf[4][j], buf[5][j]);
            });
        } else if (in_mesh) {
            visit_tape_cell(A, ci, cj, g, [&](int q) {
                add(A.x[q], A.y[q], A.lx[q], A.ly[q], A.lvx[q], A.lvy[q]);
            });
        }
        #pragma unroll
        for (int k = 0; k < NQ; ++k) s_c[k][tid] = acc[k];
        if (own_cell) A.cnt[cj * A.nx + ci] = cnt;
        __syncthreads();
        if (node_ok) {
            #pragma unroll
            for (int k = 0; k < 4; ++k) sum[k] = node_sum(s_c + 4 * k, tid);
        }
    } else if (own_cell) {
        A.cnt[cj * A.nx + ci] = 0;
    }
    if (node_ok) rev_node_update<USL>(A, node, sum[0], sum[1], sum[2], sum[3]);
}

template <bool USL>
__global__ void __launch_bounds__(TILE_THREADS, 2)
k_rev_nodal_update(const __grid_constant__ AdjStep A, const int4* __restrict__ tiles) {
    const int4 T = tiles[blockIdx.x];
    if (T.x < 0) return;   // past the listed tiles
    rev_nodal_update_tile<USL>(A, T);
}

template <bool USL>
__global__ void __launch_bounds__(TILE_THREADS, 2)
k_rev_nodal_update_batch(const AdjStep* __restrict__ table, const int4* __restrict__ tiles) {
    __shared__ AdjStep sA;
    const int4 T = tiles[blockIdx.x];
    if (T.x < 0) return;   // past the listed tiles
    load_step_args(table + T.x, sA);
    rev_nodal_update_tile<USL>(sA, T);
}

// Strain rates (xx, yy, xy) and centroid rates of a particle from the nodal
// velocities (nvx, nvy) of its cell's corners, the left-to-right sums of
// strain_rate4 with its flushes; sx, sy: signed sums + - + - of the corner
// velocities (d Gx_k / d eta and d Gy_k / d xi carry these signs).
__device__ __forceinline__ void rates_at(const int ids[4], const float Gx[4], const float Gy[4],
                                         const float Gcx[4], const float Gcy[4],
                                         const float* __restrict__ nvx, const float* __restrict__ nvy,
                                         float& r0, float& r1, float& r3, float& c0, float& c1,
                                         float& sx, float& sy) {
    float r3a = 0.0f, r3b_ = 0.0f;
    #pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float vx = nvx[ids[k]], vy = nvy[ids[k]];
        if (k == 0) {
            r0 = fm(Gx[0], vx);
            r1 = fm(Gy[0], vy);
            r3a = fm(Gx[0], vy);
            r3b_ = fm(Gy[0], vx);
            c0 = fm(Gcx[0], vx);
            c1 = fm(Gcy[0], vy);
            sx = vx;
            sy = vy;
        } else {
            r0 = fa(r0, fm(Gx[k], vx));
            r1 = fa(r1, fm(Gy[k], vy));
            r3a = fa(r3a, fm(Gx[k], vy));
            r3b_ = fa(r3b_, fm(Gy[k], vx));
            c0 = fa(c0, fm(Gcx[k], vx));
            c1 = fa(c1, fm(Gcy[k], vy));
            sx = (k & 1) ? fs(sx, vx) : fa(sx, vx);
            sy = (k & 1) ? fs(sy, vy) : fa(sy, vy);
        }
    }
    r0 = flush(r0);
    r1 = flush(r1);
    r3 = flush(fa(r3a, r3b_));
    c0 = flush(c0);
    c1 = flush(c1);
}

// Reverse of the stress update for the stress adjoint sb: the strain-rate
// adjoints (zero where the forward flushed the rate), dL/dE, the adjoint of
// the updated centroid volumetric strain (vscb) and whether the update is a
// total stress (the start-of-step stress then passes no adjoint).
//   LinearElastic, SimpleMaterial: sig' = sig + D(E) r dt;
//   Newtonian (the build's definition): sig' = K vsc' I + 2 mu dev(r) with
//   r_zz = 0, s_xy = mu r_xy (material.py has no Newtonian).
template <bool NEWT>   // NEWT: the run has Newtonian particles
__device__ __forceinline__ void stress_reverse(const MatDev& mat, float Ep, float dt, float r0, float r1,
                                               float r3, float sbxx, float sbyy, float sbzz, float sbxy,
                                               float& r0b, float& r1b, float& r3b, float& Eb,
                                               float& vscb, bool& total) {
    const float d0 = fm(r0, dt), d1 = fm(r1, dt), d3 = fm(r3, dt);
    float d0b = 0.0f, d1b = 0.0f, d3b = 0.0f;
    Eb = 0.0f;
    vscb = 0.0f;
    total = false;
    if (NEWT && mat.type == MAT_NEWTONIAN) {
        const float tr = fa(fa(sbxx, sbyy), sbzz);
        const float t3b = -fm(mat.twomu, tr);              // t3 = (r0 + r1) / 3
        vscb = fm(mat.K, tr);                              // kv = K vsc'
        const float r0n = fa(fm(mat.twomu, sbxx), fdv(t3b, 3.0f));
        const float r1n = fa(fm(mat.twomu, sbyy), fdv(t3b, 3.0f));
        r0b = r0 != 0.0f ? r0n : 0.0f;
        r1b = r1 != 0.0f ? r1n : 0.0f;
        r3b = r3 != 0.0f ? fm(mat.mu, sbxy) : 0.0f;
        total = true;
        return;
    }
    if (mat.type == MAT_LINEAR_ELASTIC) {
        float a1 = mat.a1, a2 = mat.a2, G = mat.G;
        if (Ep >= 0.0f) {
            a1 = fm(Ep, mat.c1);
            a2 = fm(Ep, mat.c2);
            G = fm(Ep, mat.c3);
        }
        d0b = fa(fa(fm(a1, sbxx), fm(a2, sbyy)), fm(a2, sbzz));
        d1b = fa(fa(fm(a2, sbxx), fm(a1, sbyy)), fm(a2, sbzz));
        d3b = fm(G, sbxy);
        Eb = fa(fa(fm(mat.c1, fa(fm(d0, sbxx), fm(d1, sbyy))),
                   fm(mat.c2, fa(fa(fm(d1, sbxx), fm(d0, sbyy)), fm(fa(d0, d1), sbzz)))),
                fm(mat.c3, fm(d3, sbxy)));
    } else if (mat.type == MAT_SIMPLE) {
        const float E = Ep >= 0.0f ? Ep : mat.E;
        d0b = fm(E, sbxx);
        d1b = fm(E, sbyy);
        d3b = fm(E, sbxy);
        Eb = fa(fa(fm(d0, sbxx), fm(d1, sbyy)), fm(d3, sbxy));
    }
    r0b = r0 != 0.0f ? fm(d0b, dt) : 0.0f;
    r1b = r1 != 0.0f ? fm(d1b, dt) : 0.0f;
    r3b = r3 != 0.0f ? fm(d3b, dt) : 0.0f;
}

// ---------------------------------------------------------------------------
// Particle velocity constraints (applied after the G2P velocity update, an
// extension): a constrained component of the end-of-step velocity is a
// constant, so its adjoint is cleared before the reverse passes.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void rev_pvc_at(const AdjStep& A, int q) {
    if (q >= A.np || !A.pvc) return;
    const uchar2 c = reinterpret_cast<const uchar2*>(A.pvc)[q];
    if (c.x) A.lvx[q] = 0.0f;
    if (c.y) A.lvy[q] = 0.0f;
}

__global__ void __launch_bounds__(PART_THREADS) k_rev_pvc(const __grid_constant__ AdjStep A) {
    rev_pvc_at(A, blockIdx.x * blockDim.x + threadIdx.x);
}

__global__ void __launch_bounds__(PART_THREADS)
k_rev_pvc_batch(const AdjStep* __restrict__ table, const int2* __restrict__ blocks) {
    __shared__ AdjStep sA;
    const int2 bm = blocks[blockIdx.x];
    load_step_args(table + bm.x, sA);
    #pragma unroll 1
    for (int k = 0; k < ADJ_ITER; ++k) rev_pvc_at(sA, (bm.y * ADJ_ITER + k) * PART_THREADS + threadIdx.x);
}

// ---------------------------------------------------------------------------
// USL pass U (before pass 1): reverse of the strain / density / stress update
// that USL runs after G2P from the updated nodal velocities vB, at the
// positions of the step start (scheme.py:127-133, particle.py:249-327).  The
// stress adjoint passes through unchanged; the strain-rate and centroid-rate
// adjoints go to pass G (their transposed gather) and to pass 2 (their
// position terms); the density adjoint becomes that of the step start.
// ---------------------------------------------------------------------------
template <bool REINIT, bool NEWT>
__device__ __forceinline__ void rev_stress_usl_at(const AdjStep& A, int q, float x, float y) {
    if (q >= A.np) return;
    int ci, cj;
    particle_cell(A, x, y, ci, cj);
    const CellGeo g = cell_geo(ci, cj, A.hx, A.hy);
    float Gx[4], Gy[4], Gcx[4], Gcy[4];
    dshape4(natural(x, g.cx, g.rx), natural(y, g.cy, g.ry), g.rx, g.ry, Gx, Gy);
    dshape4(0.0f, 0.0f, g.rx, g.ry, Gcx, Gcy);
    const int ll = cj * (A.nx + 1) + ci;
    const int ids[4] = {ll, ll + 1, ll + A.nx + 2, ll + A.nx + 1};
    float r0, r1, r3, c0, c1, sx, sy;
    rates_at(ids, Gx, Gy, Gcx, Gcy, A.nvbx, A.nvby, r0, r1, r3, c0, c1, sx, sy);
    const float dvol = fm(A.dt, fa(c0, c1));
    const float f = fa(1.0f, dvol);
    const float rho1 = fdv(A.rho[q], f);
    const MatDev& mat = A.mats[A.mat[q]];
    const float Ep = A.E ? A.E[q] : -1.0f;
    float r0b, r1b, r3b, Eb, vscb;
    bool total;
    stress_reverse<NEWT>(mat, Ep, A.dt, r0, r1, r3, A.lsxx[q], A.lsyy[q], A.lszz[q], A.lsxy[q], r0b,
                         r1b, r3b, Eb, vscb, total);
    if (total) {   // the start-of-step stress passes no adjoint (pass 2 adds the forces')
        A.lsxx[q] = 0.0f;
        A.lsyy[q] = 0.0f;
        A.lszz[q] = 0.0f;
        A.lsxy[q] = 0.0f;
    }
    const float lrho = A.lrho[q];
    float fb = -fdv(fm(lrho, rho1), f);
    if (NEWT) {   // vsc' = vsc + dvol (only Newtonian stress reads vsc; else its adjoint is 0)
        const float lvsc = fa(A.lvsc[q], vscb);
        A.lvsc[q] = lvsc;
        fb = fa(fb, lvsc);
    }
    if (!REINIT) {   // solve semantics: V' = V f carries the volume to the next step
        const float lv = A.lvol[q];
        fb = fa(fb, fm(lv, A.vol[q]));
        A.lvol[q] = fm(lv, f);
    }
    A.r0b[q] = r0b;
    A.r1b[q] = r1b;
    A.r3b[q] = r3b;
    A.c0b[q] = c0 != 0.0f ? fm(fb, A.dt) : 0.0f;
    A.c1b[q] = c1 != 0.0f ? fm(fb, A.dt) : 0.0f;
    A.lrho[q] = fdv(lrho, f);
    A.lE[q] = fa(A.lE[q], Eb);
}

template <bool REINIT, bool NEWT>
__global__ void __launch_bounds__(PART_THREADS)
k_rev_stress_usl(const __grid_constant__ AdjStep A) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < A.np) rev_stress_usl_at<REINIT, NEWT>(A, q, A.x[q], A.y[q]);
}

template <bool REINIT, bool NEWT>
__global__ void __launch_bounds__(PART_THREADS)
k_rev_stress_usl_batch(const AdjStep* __restrict__ table, const int2* __restrict__ blocks) {
    __shared__ AdjStep sA;
    const int2 bm = blocks[blockIdx.x];
    load_step_args(table + bm.x, sA);
    #pragma unroll 1
    for (int k = 0; k < ADJ_ITER; ++k) {
        const int q = (bm.y * ADJ_ITER + k) * PART_THREADS + threadIdx.x;
        if (q < sA.np) rev_stress_usl_at<REINIT, NEWT>(sA, q, sA.x[q], sA.y[q]);
    }
}

// ---------------------------------------------------------------------------
// Pass 2: reverse of the forces (element.py:236-268, 842-901) and, for USF,
// of the strain / volume / stress update before them (particle.py:249-327,
// material.py:113-131).  USL forces use the start-of-step stress and the
// reset volume V0; the strain-rate adjoints of its later stress update come
// from pass U and only add their position terms here.
// ---------------------------------------------------------------------------
template <bool USL, bool TRAC, bool REINIT, bool NEWT>
__device__ __forceinline__ void rev_forces_at(const AdjStep& A, int q, float x, float y) {
    if (q >= A.np) return;
    int ci, cj;
    particle_cell(A, x, y, ci, cj);
    const CellGeo g = cell_geo(ci, cj, A.hx, A.hy);
    const float xi = natural(x, g.cx, g.rx), eta = natural(y, g.cy, g.ry);
    float N[4], Gx[4], Gy[4];
    shape4(xi, eta, N);
    dshape4(xi, eta, g.rx, g.ry, Gx, Gy);
    const int ll = cj * (A.nx + 1) + ci;
    const int ids[4] = {ll, ll + 1, ll + A.nx + 2, ll + A.nx + 1};
    // V0: the volume at the step start (the per-step set-up V_el / count, or
    // under solve semantics the carried volume); m: the particle mass
    float V0;
    if (REINIT) {
        const int cnt = A.cnt[cj * A.nx + ci];
        V0 = cnt ? fdv(A.vol_el, (float)cnt) : 0.0f;
    } else {
        V0 = A.vol[q];
    }
    const float rho0 = A.rho[q];
    const float m = REINIT ? fm(V0, rho0) : A.mass[q];

    // the stress and volume of the forces: USF recomputes the strain rates
    // from vA and the stress update; sAx, sAy: signed sums of the corner
    // velocities the strain rates used (vA for USF, vB for USL)
    float r0 = 0.0f, r1 = 0.0f, r3 = 0.0f, c0 = 0.0f, c1 = 0.0f, sAx = 0.0f, sAy = 0.0f;
    PState p{};
    p.sxx = A.sxx[q];
    p.syy = A.syy[q];
    p.szz = A.szz[q];
    p.sxy = A.sxy[q];
    p.rho = rho0;
    p.vsc = NEWT ? A.vsc[q] : 0.0f;   // taped when a material uses it (Newtonian)
    float f = 1.0f, V = V0;
    const MatDev& mat = A.mats[A.mat[q]];
    const float Ep = A.E ? A.E[q] : -1.0f;
    if (!USL) {
        float Gcx[4], Gcy[4];
        dshape4(0.0f, 0.0f, g.rx, g.ry, Gcx, Gcy);
        rates_at(ids, Gx, Gy, Gcx, Gcy, A.nvax, A.nvay, r0, r1, r3, c0, c1, sAx, sAy);
        const float dvol = fm(A.dt, fa(c0, c1));
        f = strain_stress_update(mat, Ep, A.dt, r0, r1, r3, dvol, p);
        V = fm(V0, f);
    }

    // particle tractions t_d = f(t) tau_d V / size0 (mesh.py:60-77,
    // particle.py:329-343, element.py:286-303): t_d and d t_d / dV
    float trx = 0.0f, try_ = 0.0f, tqx = 0.0f, tqy = 0.0f;
    if (TRAC && A.tr_fn) {
        const float tt = step_time(A.step, A.dt);
        const float size0 = REINIT ? sqrtf(V0) : A.psize[q];
        #pragma unroll
        for (int d = 0; d < 2; ++d) {
            const int code = A.tr_fn[2 * q + d];
            if (!code) continue;
            const float tv = fm(fn_value(A, code, tt), A.tr_tau[2 * q + d]);
            const float tr = fdv(fm(tv, V), size0), tq = fdv(tv, size0);
            if (d == 0) {
                trx = tr;
                tqx = tq;
            } else {
                try_ = tr;
                tqy = tq;
            }
        }
    }

    // G2P, external and internal forces: adjoints of the shape functions (as
    // x-bar, y-bar contributions), of m and V, of the stress the forces used,
    // and the signed sums of the gradient adjoints
    float gx, gy, hx, hy;
    g2p_seeds(A, q, gx, gy, hx, hy);
    float xb = A.lx[q], yb = A.ly[q];
    float mb = 0.0f, Vb = 0.0f, fsxx = 0.0f, fsyy = 0.0f, fsxy = 0.0f, sgx = 0.0f, sgy = 0.0f;
    #pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int n = ids[k];
        const float fbx = A.fbx[n], fby = A.fby[n];
        const float vBx = A.nvbx[n], vBy = A.nvby[n];
        const float fg = fa(fm(fbx, A.gx), fm(fby, A.gy));   // F-bar . g
        float Nb = fa(fa(fa(fm(gx, vBx), fm(gy, vBy)), fa(fm(hx, A.nax[n]), fm(hy, A.nay[n]))),
                      fm(m, fg));
        if (TRAC) {
            Nb = fa(Nb, fa(fm(fbx, trx), fm(fby, try_)));   // F-bar . traction
            if (!USL || !REINIT) Vb = fa(Vb, fm(N[k], fa(fm(fbx, tqx), fm(fby, tqy))));
        }
        if (USL) {
            sAx = k == 0 ? vBx : (k & 1) ? fs(sAx, vBx) : fa(sAx, vBx);
            sAy = k == 0 ? vBy : (k & 1) ? fs(sAy, vBy) : fa(sAy, vBy);
        }
        mb = fa(mb, fm(N[k], fg));
        const float fx = fa(fm(Gx[k], p.sxx), fm(Gy[k], p.sxy));
        const float fy = fa(fm(Gy[k], p.syy), fm(Gx[k], p.sxy));
        if (!USL || !REINIT) Vb = fs(Vb, fa(fm(fbx, fx), fm(fby, fy)));
        fsxx = fa(fsxx, fm(fbx, Gx[k]));
        fsyy = fa(fsyy, fm(fby, Gy[k]));
        fsxy = fa(fsxy, fa(fm(fbx, Gy[k]), fm(fby, Gx[k])));
        const float gxk = -fm(V, fa(fm(fbx, p.sxx), fm(fby, p.sxy)));
        const float gyk = -fm(V, fa(fm(fbx, p.sxy), fm(fby, p.syy)));
        sgx = (k & 1) ? fs(sgx, gxk) : fa(sgx, gxk);
        sgy = (k & 1) ? fs(sgy, gyk) : fa(sgy, gyk);
        xb = fa(xb, fm(Nb, Gx[k]));
        yb = fa(yb, fm(Nb, Gy[k]));
    }
    // stress adjoint: loss/next-step part (through pass U for USL) + force part
    float sbxx = fs(A.lsxx[q], fm(V, fsxx));
    float sbyy = fs(A.lsyy[q], fm(V, fsyy));
    float sbzz = A.lszz[q];
    float sbxy = fs(A.lsxy[q], fm(V, fsxy));

    float r0b, r1b, r3b, rhob;
    if (USL) {
        r0b = A.r0b[q];
        r1b = A.r1b[q];
        r3b = A.r3b[q];
        rhob = REINIT ? fa(A.lrho[q], fm(V0, mb)) : A.lrho[q];
        if (!REINIT) A.lvol[q] = fa(A.lvol[q], Vb);   // the forces used the start volume
    } else {
        float Eb, vscb;
        bool total;
        stress_reverse<NEWT>(mat, Ep, A.dt, r0, r1, r3, sbxx, sbyy, sbzz, sbxy, r0b, r1b, r3b, Eb, vscb,
                             total);
        if (total) sbxx = sbyy = sbzz = sbxy = 0.0f;   // total stress: no adjoint to the start
        // reverse of V = V0 (1 + dvol), rho' = rho / (1 + dvol), m = V0 rho,
        // vsc' = vsc + dvol (solve semantics: m is constant and V also
        // carries to the next step)
        const float lrho = A.lrho[q];
        const float Vt = REINIT ? Vb : fa(Vb, A.lvol[q]);
        float fb = fs(fm(Vt, V0), fdv(fm(lrho, p.rho), f));
        if (NEWT) {   // only Newtonian stress reads vsc; otherwise its adjoint is 0
            const float lvsc = fa(A.lvsc[q], vscb);
            A.lvsc[q] = lvsc;
            fb = fa(fb, lvsc);
        }
        rhob = REINIT ? fa(fdv(lrho, f), fm(V0, mb)) : fdv(lrho, f);
        if (!REINIT) A.lvol[q] = fm(Vt, f);
        A.lE[q] = fa(A.lE[q], Eb);
        A.r0b[q] = r0b;
        A.r1b[q] = r1b;
        A.r3b[q] = r3b;
        A.c0b[q] = c0 != 0.0f ? fm(fb, A.dt) : 0.0f;
        A.c1b[q] = c1 != 0.0f ? fm(fb, A.dt) : 0.0f;
    }

    // strain-rate part of the gradient adjoints: Gx_k-bar += r0b v_x,k + r3b
    // v_y,k, Gy_k-bar += r1b v_y,k + r3b v_x,k; their signed sums move x, y
    sgx = fa(sgx, fa(fm(r0b, sAx), fm(r3b, sAy)));
    sgy = fa(sgy, fa(fm(r1b, sAy), fm(r3b, sAx)));
    const float rxy = fm(fm(0.25f, g.rx), g.ry);
    xb = fa(xb, fm(rxy, sgy));
    yb = fa(yb, fm(rxy, sgx));

    A.lx[q] = xb;
    A.ly[q] = yb;
    A.lsxx[q] = sbxx;
    A.lsyy[q] = sbyy;
    A.lszz[q] = sbzz;
    A.lsxy[q] = sbxy;
    A.lrho[q] = rhob;
}

template <bool USL, bool TRAC, bool REINIT, bool NEWT>
__global__ void __launch_bounds__(PART_THREADS, 4)
k_rev_forces(const __grid_constant__ AdjStep A) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < A.np) rev_forces_at<USL, TRAC, REINIT, NEWT>(A, q, A.x[q], A.y[q]);
}

template <bool USL, bool TRAC, bool REINIT, bool NEWT>
__global__ void __launch_bounds__(PART_THREADS, 4)
k_rev_forces_batch(const AdjStep* __restrict__ table, const int2* __restrict__ blocks) {
    __shared__ AdjStep sA;
    const int2 bm = blocks[blockIdx.x];
    load_step_args(table + bm.x, sA);
    #pragma unroll 1
    for (int k = 0; k < ADJ_ITER; ++k) {
        const int q = (bm.y * ADJ_ITER + k) * PART_THREADS + threadIdx.x;
        if (q < sA.np) rev_forces_at<USL, TRAC, REINIT, NEWT>(sA, q, sA.x[q], sA.y[q]);
    }
}

// ---------------------------------------------------------------------------
// Pass 3: transposed strain-rate gather (vA-bar += sum over particles of
// G r-bar + Gc c-bar) and the reverse nodal velocity vA = C(flush(P / M)),
// P = flush(sum N m v) (element.py:191-202, 331-334; particle.py:281-313).
// The same tile kernel is USL's pass G (the gather alone, of the pass-U
// adjoints, into vabx, vaby); USL's pass 3 has no gather.
// ---------------------------------------------------------------------------
enum RevKinMode { RK_USF, RK_GATHER, RK_NODES };
__device__ __forceinline__ void rev_node_velocity(const AdjStep& A, int n, float vbx, float vby) {
    float qbx = 0.0f, qby = 0.0f, mbt = A.mb[n];
    const float M = A.nm[n];
    if (M != 0.0f) {
        const uint16_t code = A.ncons[n];
        const bool cx = (code & 0xff) != 0, cy = (code >> 8) != 0;
        const float vAx = A.nvax[n], vAy = A.nvay[n];
        const float ubx = (cx || vAx == 0.0f) ? 0.0f : vbx;
        const float uby = (cy || vAy == 0.0f) ? 0.0f : vby;
        qbx = fdv(ubx, M);
        qby = fdv(uby, M);
        mbt = fs(mbt, fdv(fa(fm(ubx, vAx), fm(uby, vAy)), M));
    }
    A.qbx[n] = qbx;
    A.qby[n] = qby;
    A.mbt[n] = mbt;
}

template <int MODE>
__device__ __forceinline__ void rev_nodal_kinematics_tile(const AdjStep& A, const int4 T) {
    constexpr int NQ = 8;    // [vA-bar x, y] x corner
    __shared__ float s_c[NQ][SC_STRIDE];
    __shared__ __align__(16) float s_row[TILE_CY][7][REV_ROW_P];
    __shared__ int s_cs[TILE_CY][33];
    const int tid = threadIdx.x, tx = tid % TILE_CX, ty = tid / TILE_CX;
    const int c0x = T.y * TILE_NX - 1, c0y = T.z * TILE_NY - 1;
    const int ci = c0x + tx, cj = c0y + ty;
    const bool node_ok = tx < TILE_NX && ty < TILE_NY && c0x + 1 + tx <= A.nx && c0y + 1 + ty <= A.ny;
    const int node = (c0y + 1 + ty) * (A.nx + 1) + c0x + 1 + tx;
    float sx = 0.0f, sy = 0.0f;
    int L_cs, L_cs32, L_occ, L_drift;
    rev_tile_loads(A, c0x, c0y, cj, tx, L_cs, L_cs32, L_occ, L_drift);
    s_cs[ty][tx] = L_cs;
    if (tx == 0) s_cs[ty][32] = L_cs32;
    if (__syncthreads_or(L_occ)) {
        const bool slow = __syncthreads_or(L_drift) != 0;
        const bool in_mesh = ci >= 0 && ci < A.nx && cj >= 0 && cj < A.ny;
        const CellGeo g = cell_geo(ci, cj, A.hx, A.hy);
        float Gcx[4], Gcy[4];
        dshape4(0.0f, 0.0f, g.rx, g.ry, Gcx, Gcy);
        float acc[NQ];
        #pragma unroll
        for (int k = 0; k < NQ; ++k) acc[k] = 0.0f;
        auto add = [&](float x, float y, float r0b, float r1b, float r3b, float c0b, float c1b) {
            float Gx[4], Gy[4];
            dshape4(natural(x, g.cx, g.rx), natural(y, g.cy, g.ry), g.rx, g.ry, Gx, Gy);
            #pragma unroll
            for (int k = 0; k < 4; ++k) {
                acc[k] = fa(acc[k], fa(fa(fm(Gx[k], r0b), fm(Gy[k], r3b)), fm(Gcx[k], c0b)));
                acc[4 + k] = fa(acc[4 + k], fa(fa(fm(Gy[k], r1b), fm(Gx[k], r3b)), fm(Gcy[k], c1b)));
            }
        };
        if (!slow) {
            const int* cs = s_cs[ty];
            const float* const src[7] = {A.x, A.y, A.r0b, A.r1b, A.r3b, A.c0b, A.c1b};
            float (*buf)[REV_ROW_P] = s_row[ty];
            row_pass16<7, REV_ROW_P>(buf, src, cs[0], cs[32], cs[tx], cs[tx + 1], tx, [&](int, int j) {
                add(buf[0][j], buf[1][j], buf[2][j], buf[3][j], buf[4][j], buf[5][j], buf[6][j]);
            });
        } else if (in_mesh) {
            visit_tape_cell(A, ci, cj, g, [&](int q) {
                add(A.x[q], A.y[q], A.r0b[q], A.r1b[q], A.r3b[q], A.c0b[q], A.c1b[q]);
            });
        }
        #pragma unroll
        for (int k = 0; k < NQ; ++k) s_c[k][tid] = acc[k];
        __syncthreads();
        if (node_ok) {
            sx = node_sum(s_c + 0, tid);
            sy = node_sum(s_c + 4, tid);
        }
    }
    if (!node_ok) return;
    if (MODE == RK_GATHER) {
        A.vabx[node] = sx;
        A.vaby[node] = sy;
    } else {
        rev_node_velocity(A, node, fa(A.vabx[node], sx), fa(A.vaby[node], sy));
    }
}

// USL pass 3: the reverse nodal velocity of the tile's nodes from vA-bar alone.
__device__ __forceinline__ void rev_node_velocity_tile(const AdjStep& A, const int4 T) {
    const int tid = threadIdx.x, tx = tid % TILE_CX, ty = tid / TILE_CX;
    const int c0x = T.y * TILE_NX - 1, c0y = T.z * TILE_NY - 1;
    if (tx < TILE_NX && ty < TILE_NY && c0x + 1 + tx <= A.nx && c0y + 1 + ty <= A.ny) {
        const int node = (c0y + 1 + ty) * (A.nx + 1) + c0x + 1 + tx;
        rev_node_velocity(A, node, A.vabx[node], A.vaby[node]);
    }
}

template <int MODE>
__global__ void __launch_bounds__(TILE_THREADS, 2)
k_rev_nodal_kinematics(const __grid_constant__ AdjStep A, const int4* __restrict__ tiles) {
    const int4 T = tiles[blockIdx.x];
    if (T.x < 0) return;   // past the listed tiles
    if (MODE == RK_NODES) rev_node_velocity_tile(A, T);
    else rev_nodal_kinematics_tile<MODE>(A, T);
}

template <int MODE>
__global__ void __launch_bounds__(TILE_THREADS, 2)
k_rev_nodal_kinematics_batch(const AdjStep* __restrict__ table, const int4* __restrict__ tiles) {
    __shared__ AdjStep sA;
    const int4 T = tiles[blockIdx.x];
    if (T.x < 0) return;   // past the listed tiles
    load_step_args(table + T.x, sA);
    if (MODE == RK_NODES) rev_node_velocity_tile(sA, T);
    else rev_nodal_kinematics_tile<MODE>(sA, T);
}

// ---------------------------------------------------------------------------
// Pass 4: reverse of the mass and momentum P2G (element.py:122-189) and of
// m = V0 rho (particle.py:158-178).
// ---------------------------------------------------------------------------
template <bool REINIT>
__device__ __forceinline__ void rev_mass_momentum_at(const AdjStep& A, int q, float x, float y) {
    if (q >= A.np) return;
    int ci, cj;
    particle_cell(A, x, y, ci, cj);
    const CellGeo g = cell_geo(ci, cj, A.hx, A.hy);
    const float xi = natural(x, g.cx, g.rx), eta = natural(y, g.cy, g.ry);
    float N[4], Gx[4], Gy[4];
    shape4(xi, eta, N);
    dshape4(xi, eta, g.rx, g.ry, Gx, Gy);
    const int ll = cj * (A.nx + 1) + ci;
    const int ids[4] = {ll, ll + 1, ll + A.nx + 2, ll + A.nx + 1};
    float V0 = 0.0f, m;
    if (REINIT) {
        const int cnt = A.cnt[cj * A.nx + ci];
        V0 = cnt ? fdv(A.vol_el, (float)cnt) : 0.0f;
        m = fm(V0, A.rho[q]);
    } else {
        m = A.mass[q];   // solve semantics: constant mass
    }
    const float vx = A.vx[q], vy = A.vy[q];
    float mb = 0.0f, sqx = 0.0f, sqy = 0.0f, xb = A.lx[q], yb = A.ly[q];
    #pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float qx = A.qbx[ids[k]], qy = A.qby[ids[k]];
        const float t = fa(fa(fm(qx, vx), fm(qy, vy)), A.mbt[ids[k]]);
        mb = fa(mb, fm(N[k], t));
        sqx = fa(sqx, fm(N[k], qx));
        sqy = fa(sqy, fm(N[k], qy));
        const float nb = fm(m, t);
        xb = fa(xb, fm(nb, Gx[k]));
        yb = fa(yb, fm(nb, Gy[k]));
    }
    const float lvx = A.velocity_update ? 0.0f : A.lvx[q];
    const float lvy = A.velocity_update ? 0.0f : A.lvy[q];
    A.lvx[q] = fa(lvx, fm(m, sqx));
    A.lvy[q] = fa(lvy, fm(m, sqy));
    if (REINIT) A.lrho[q] = fa(A.lrho[q], fm(V0, mb));
    A.lx[q] = xb;
    A.ly[q] = yb;
}

template <bool REINIT>
__global__ void __launch_bounds__(PART_THREADS)
k_rev_mass_momentum(const __grid_constant__ AdjStep A) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < A.np) rev_mass_momentum_at<REINIT>(A, q, A.x[q], A.y[q]);
}

template <bool REINIT>
__global__ void __launch_bounds__(PART_THREADS)
k_rev_mass_momentum_batch(const AdjStep* __restrict__ table, const int2* __restrict__ blocks) {
    __shared__ AdjStep sA;
    const int2 bm = blocks[blockIdx.x];
    load_step_args(table + bm.x, sA);
    // the positions of all the block's chunks in flight at once
    float x[ADJ_ITER], y[ADJ_ITER];
    #pragma unroll
    for (int k = 0; k < ADJ_ITER; ++k) {
        const int q = (bm.y * ADJ_ITER + k) * PART_THREADS + threadIdx.x;
        x[k] = q < sA.np ? sA.x[q] : 0.0f;
        y[k] = q < sA.np ? sA.y[q] : 0.0f;
    }
    #pragma unroll
    for (int k = 0; k < ADJ_ITER; ++k)
        rev_mass_momentum_at<REINIT>(sA, (bm.y * ADJ_ITER + k) * PART_THREADS + threadIdx.x, x[k], y[k]);
}

// table[i] = bases[i] with the tape pointers moved to slot t.
__global__ void k_adj_table(const AdjStep* __restrict__ bases, int n, int t,
                            AdjStep* __restrict__ table) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    AdjStep a = bases[i];
    const size_t op = (size_t)t * a.sp, on = (size_t)t * a.sn, oc = (size_t)t * a.sc;
    a.x += op; a.y += op; a.vx += op; a.vy += op;
    a.sxx += op; a.syy += op; a.szz += op; a.sxy += op; a.rho += op;
    if (a.vol) a.vol += op;
    if (a.vsc) a.vsc += op;
    a.cflag += oc;
    a.nm += on; a.nvax += on; a.nvay += on; a.nvbx += on; a.nvby += on; a.nax += on; a.nay += on;
    a.step += t;
    table[i] = a;
}

inline int blocks_for(int n, int t) { return (n + t - 1) / t; }

}  // namespace

namespace {

// The particle passes of one reverse step for a configuration: pass U (USL,
// `first`) or pass 2, single-simulation and batched launches.
template <bool USL, bool TRAC, bool REINIT, bool NEWT>
void rev_particles(const AdjStep& A, const AdjStep* table, const int2* pbk, int nb, bool first,
                   cudaStream_t s) {
    if (table) {
        if (first) {
            if (USL) k_rev_stress_usl_batch<REINIT, NEWT><<<nb, PART_THREADS, 0, s>>>(table, pbk);
        } else {
            k_rev_forces_batch<USL, TRAC, REINIT, NEWT><<<nb, PART_THREADS, 0, s>>>(table, pbk);
        }
    } else {
        if (first) {
            if (USL) k_rev_stress_usl<REINIT, NEWT><<<nb, PART_THREADS, 0, s>>>(A);
        } else {
            k_rev_forces<USL, TRAC, REINIT, NEWT><<<nb, PART_THREADS, 0, s>>>(A);
        }
    }
}

using RevParticlesFn = void (*)(const AdjStep&, const AdjStep*, const int2*, int, bool, cudaStream_t);
#define MPM_REV(u, t, r) rev_particles<u, t, r, false>, rev_particles<u, t, r, true>
constexpr RevParticlesFn kRevParticles[16] = {
    MPM_REV(false, false, false), MPM_REV(false, false, true), MPM_REV(false, true, false),
    MPM_REV(false, true, true),   MPM_REV(true, false, false), MPM_REV(true, false, true),
    MPM_REV(true, true, false),   MPM_REV(true, true, true)};
#undef MPM_REV

struct RevConfig {
    bool usl, trac, reinit, newt;
    RevParticlesFn fn() const { return kRevParticles[usl * 8 + trac * 4 + reinit * 2 + newt]; }
};

void rev_part(const AdjStep& A, const RevConfig& c, int pb, bool first, cudaStream_t s) {
    c.fn()(A, nullptr, nullptr, pb, first, s);
}
void rev_part_batch(const AdjStep* t, const RevConfig& c, const int2* pbk, int npb, bool first,
                    cudaStream_t s) {
    static const AdjStep unused{};   // the batched launches read the device table `t`
    c.fn()(unused, t, pbk, npb, first, s);
}
}  // namespace

cudaError_t launch_rev_step(const AdjStep& A, bool usl, bool trac, const int4* tiles, int ntiles,
                            cudaStream_t s) {
    const int pb = A.np > 0 ? blocks_for(A.np, PART_THREADS) : 0;
    const bool reinit = A.reinit != 0;
    const RevConfig rc{usl, trac, reinit, A.vsc != nullptr};
    if (A.pvc && pb) k_rev_pvc<<<pb, PART_THREADS, 0, s>>>(A);
    if (usl) {
        if (pb) rev_part(A, rc, pb, true, s);
        if (ntiles > 0) k_rev_nodal_kinematics<RK_GATHER><<<ntiles, TILE_THREADS, 0, s>>>(A, tiles);
        if (ntiles > 0) k_rev_nodal_update<true><<<ntiles, TILE_THREADS, 0, s>>>(A, tiles);
        if (pb) rev_part(A, rc, pb, false, s);
        if (ntiles > 0) k_rev_nodal_kinematics<RK_NODES><<<ntiles, TILE_THREADS, 0, s>>>(A, tiles);
    } else {
        if (ntiles > 0) k_rev_nodal_update<false><<<ntiles, TILE_THREADS, 0, s>>>(A, tiles);
        if (pb) rev_part(A, rc, pb, false, s);
        if (ntiles > 0) k_rev_nodal_kinematics<RK_USF><<<ntiles, TILE_THREADS, 0, s>>>(A, tiles);
    }
    if (pb) {
        if (reinit) k_rev_mass_momentum<true><<<pb, PART_THREADS, 0, s>>>(A);
        else k_rev_mass_momentum<false><<<pb, PART_THREADS, 0, s>>>(A);
    }
    return cudaGetLastError();
}

cudaError_t launch_adj_table(const AdjStep* bases, int n, int t, AdjStep* table, cudaStream_t s) {
    if (n > 0) k_adj_table<<<blocks_for(n, 128), 128, 0, s>>>(bases, n, t, table);
    return cudaGetLastError();
}

cudaError_t launch_rev_batch(const AdjStep* table, bool usl, bool trac, bool pvc, bool reinit, bool newt,
                             const int4* tiles, int ntiles, const int2* part_blocks, int n_part_blocks,
                             cudaStream_t s) {
    const int nt = ntiles, npb = n_part_blocks;
    const RevConfig rc{usl, trac, reinit, newt};
    if (pvc && npb > 0) k_rev_pvc_batch<<<npb, PART_THREADS, 0, s>>>(table, part_blocks);
    if (usl) {
        if (npb > 0) rev_part_batch(table, rc, part_blocks, npb, true, s);
        if (nt > 0) k_rev_nodal_kinematics_batch<RK_GATHER><<<nt, TILE_THREADS, 0, s>>>(table, tiles);
        if (nt > 0) k_rev_nodal_update_batch<true><<<nt, TILE_THREADS, 0, s>>>(table, tiles);
        if (npb > 0) rev_part_batch(table, rc, part_blocks, npb, false, s);
        if (nt > 0) k_rev_nodal_kinematics_batch<RK_NODES><<<nt, TILE_THREADS, 0, s>>>(table, tiles);
    } else {
        if (nt > 0) k_rev_nodal_update_batch<false><<<nt, TILE_THREADS, 0, s>>>(table, tiles);
        if (npb > 0) rev_part_batch(table, rc, part_blocks, npb, false, s);
        if (nt > 0) k_rev_nodal_kinematics_batch<RK_USF><<<nt, TILE_THREADS, 0, s>>>(table, tiles);
    }
    if (npb > 0) {
        if (reinit) k_rev_mass_momentum_batch<true><<<npb, PART_THREADS, 0, s>>>(table, part_blocks);
        else k_rev_mass_momentum_batch<false><<<npb, PART_THREADS, 0, s>>>(table, part_blocks);
    }
    return cudaGetLastError();
}

}  // namespace mpm
