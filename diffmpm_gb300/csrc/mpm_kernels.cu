// Kernels of the explicit MPM step on GB300 (sm_103a).
//
// Work decomposition.  The mesh is cut into tiles of 31 x 15 nodes.  One CTA
// of 512 threads (16 warps, one warp per cell row) handles one tile: thread
// (lx, ly) owns cell (31 tx - 1 + lx, 15 ty - 1 + ly), so a CTA covers the
// 32 x 16 cells that touch its 31 x 15 owned nodes.  The nodes of a tile are
// written by that CTA only; particles are written by the CTA owning their
// current cell (P2G phases) or their sort-cell (G2P).  No floating-point
// atomics are used: every nodal sum is formed in a fixed order (particles of a
// cell in storage order, then the four cells around the node), so results are
// bitwise reproducible for a given re-sort schedule.
//
// Particles are stored sorted by the cell they were in at the last re-sort
// (their sort-cell).  Between re-sorts a particle may drift to a neighbouring
// cell; a thread gathering the particles of cell c scans its own sort-cell and
// the neighbouring sort-cells whose drift flag is set.  A particle that drifts
// two cells away sets ST_DRIFT_VIOLATION and the host rolls the block back.
#include <cuda_runtime.h>
#include <cstdint>
#include "mpm_device.cuh"
#include "mpm_kernels.h"

namespace mpm {

__device__ __forceinline__ int load_step(const Control* ctl) {
    return *reinterpret_cast<const volatile int*>(&ctl->step);
}

// Visit, in a fixed order, the particles whose current cell is (ci, cj):
// sort-cells (ci+di, cj+dj) row by row; a neighbour is scanned only when its
// drift flag is set, and particles of a flagged sort-cell are tested.
template <class F>
__device__ __forceinline__ void visit_cell(const SimDev& S, int ci, int cj, const CellGeo& g,
                                           F&& f) {
    const int nx = S.nx, ny = S.ny;
    #pragma unroll 1
    for (int dj = -1; dj <= 1; ++dj) {
        const int sj = cj + dj;
        if (sj < 0 || sj >= ny) continue;
        #pragma unroll 1
        for (int di = -1; di <= 1; ++di) {
            const int si = ci + di;
            if (si < 0 || si >= nx) continue;
            const int s = sj * nx + si;
            const bool flagged = S.cflag[s] != 0;
            if (!(di == 0 && dj == 0) && !flagged) continue;
            const int b = S.cstart[s], e = S.cstart[s + 1];
            #pragma unroll 1
            for (int q = b; q < e; ++q) {
                if (flagged && !in_cell(g, S.x[q], S.y[q])) continue;
                f(q);
            }
        }
    }
}

__device__ __forceinline__ int count_cell(const SimDev& S, int ci, int cj, const CellGeo& g) {
    int n = 0;
    visit_cell(S, ci, cj, g, [&](int) { ++n; });
    return n;
}

__device__ __forceinline__ void cell_nodes(const SimDev& S, int ci, int cj, int ids[4]) {
    const int ll = cj * (S.nx + 1) + ci;
    ids[0] = ll;
    ids[1] = ll + 1;
    ids[2] = ll + S.nx + 2;
    ids[3] = ll + S.nx + 1;
}

// Sum of the four cell-corner partials meeting at the node of thread `tid`
// (node = lower-left corner of cell tid + 33): cell (I-1,J-1) corner 2,
// cell (I,J-1) corner 3, cell (I-1,J) corner 1, cell (I,J) corner 0.
__device__ __forceinline__ float node_sum(const float (*s)[TILE_THREADS], int tid) {
    return fa(fa(fa(s[2][tid], s[3][tid + 1]), s[1][tid + TILE_CX]), s[0][tid + TILE_CX + 1]);
}

__device__ __forceinline__ void apply_constraint(const SimDev& S, uint16_t code, float& vx,
                                                 float& vy, float* ax, float* ay) {
    const int c0 = code & 0xff, c1 = code >> 8;
    if (c0) {
        vx = S.cons_vel[c0 - 1];
        if (ax) *ax = 0.0f;
    }
    if (c1) {
        vy = S.cons_vel[c1 - 1];
        if (ay) *ay = 0.0f;
    }
}

// ---------------------------------------------------------------------------
// Phase 1: nodal kinematics (diffmpm/scheme.py:22-29) with the step's volume
// set-up (diffmpm/solver.py:81-85 via tree_unflatten, solver.py:100-111).
//   P2G of mass and momentum (element.py:122-189), nodal velocity
//   (element.py:191-202), velocity constraints (element.py:331-334).
// ---------------------------------------------------------------------------
template <bool REINIT>
__global__ void __launch_bounds__(TILE_THREADS)
k_nodal_kinematics(const SimDev* __restrict__ sims, const int4* __restrict__ tiles,
                   Control* __restrict__ ctl) {
    __shared__ float s_m[4][TILE_THREADS];
    __shared__ float s_px[4][TILE_THREADS];
    __shared__ float s_py[4][TILE_THREADS];
    const int4 T = tiles[blockIdx.x];
    const SimDev& S = sims[T.x];
    const int parity = load_step(ctl) & 1;
    const int tid = threadIdx.x, lx = tid & (TILE_CX - 1), ly = tid / TILE_CX;
    const int c0x = T.y * TILE_NX - 1, c0y = T.z * TILE_NY - 1;
    const int ci = c0x + lx, cj = c0y + ly;

    float m[4] = {0.f, 0.f, 0.f, 0.f}, px[4] = {0.f, 0.f, 0.f, 0.f}, py[4] = {0.f, 0.f, 0.f, 0.f};
    if (ci >= 0 && ci < S.nx && cj >= 0 && cj < S.ny) {
        const CellGeo g = cell_geo(ci, cj, S.hx, S.hy);
        const float* __restrict__ rho = S.rho[parity];
        float V0 = 0.0f;
        if (REINIT) {
            const int cnt = count_cell(S, ci, cj, g);
            if (cnt) V0 = fdv(S.vol_el, (float)cnt);   // particle.py:169-178
        }
        visit_cell(S, ci, cj, g, [&](int q) {
            const float mp = REINIT ? fm(V0, rho[q]) : S.mass[q];
            const float xi = natural(S.x[q], g.cx, g.rx);
            const float eta = natural(S.y[q], g.cy, g.ry);
            float N[4];
            shape4(xi, eta, N);
            const float pvx = fm(mp, S.vx[q]), pvy = fm(mp, S.vy[q]);
            #pragma unroll
            for (int k = 0; k < 4; ++k) {
                m[k] = fa(m[k], fm(mp, N[k]));
                px[k] = fa(px[k], fm(N[k], pvx));
                py[k] = fa(py[k], fm(N[k], pvy));
            }
        });
    }
    #pragma unroll
    for (int k = 0; k < 4; ++k) {
        s_m[k][tid] = m[k];
        s_px[k][tid] = px[k];
        s_py[k][tid] = py[k];
    }
    __syncthreads();
    if (lx < TILE_NX && ly < TILE_NY) {
        const int I = c0x + 1 + lx, J = c0y + 1 + ly;
        if (I <= S.nx && J <= S.ny) {
            const int n = J * (S.nx + 1) + I;
            const float mass = node_sum(s_m, tid);
            const float pxn = flush(node_sum(s_px, tid));
            const float pyn = flush(node_sum(s_py, tid));
            float vx, vy;
            if (mass == 0.0f) {
                vx = S.nvbx[n];
                vy = S.nvby[n];
            } else {
                vx = fdv(pxn, mass);
                vy = fdv(pyn, mass);
            }
            vx = flush(vx);
            vy = flush(vy);
            apply_constraint(S, S.ncons[n], vx, vy, nullptr, nullptr);
            S.nm[n] = mass;
            S.nvax[n] = vx;
            S.nvay[n] = vy;
        }
    }
}

// Particle traction t_p[d] = f(t) tau_d V / size (diffmpm/mesh.py:60-77,
// particle.py:329-343), accumulated into the body-force partials.
template <bool TRAC>
__device__ __forceinline__ void add_traction(const SimDev& S, int q, float t, float V, float size,
                                             const float N[4], float fex[4], float fey[4]) {
    if constexpr (TRAC) {
    #pragma unroll
    for (int d = 0; d < 2; ++d) {
        const int code = S.tr_fn[2 * q + d];
        if (!code) continue;
        const float tv = fm(fn_value(S, code, t), S.tr_tau[2 * q + d]);
        const float tr = fdv(fm(tv, V), size);
        #pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (d == 0) fex[k] = fa(fex[k], fm(N[k], tr));
            else fey[k] = fa(fey[k], fm(N[k], tr));
        }
    }
    }
}

// Nodal update shared by both schemes: concentrated forces (element.py:270-284),
// a = nan_to_num(f/m), v += a dt, constraints, flush (element.py:305-329).
__device__ __forceinline__ void nodal_update(const SimDev& S, int n, float t, float fix, float fiy,
                                             float fex, float fey) {
    if (S.cnf_ptr) {
        const int b = S.cnf_ptr[n], e = S.cnf_ptr[n + 1];
        #pragma unroll 1
        for (int k = b; k < e; ++k) {
            const float val = fm(fn_value(S, S.cnf_fn[k], t), S.cnf_val[k]);
            if (S.cnf_dir[k] == 0) fex = fa(fex, val);
            else fey = fa(fey, val);
        }
    }
    const float tx = fa(fa(fix, fex), 0.0f);
    const float ty = fa(fa(fiy, fey), 0.0f);
    const float mass = S.nm[n];
    float ax = nan_to_num(fdv(tx, mass));
    float ay = nan_to_num(fdv(ty, mass));
    float vx = fa(S.nvax[n], fm(ax, S.dt));
    float vy = fa(S.nvay[n], fm(ay, S.dt));
    apply_constraint(S, S.ncons[n], vx, vy, &ax, &ay);
    S.nvbx[n] = flush(vx);
    S.nvby[n] = flush(vy);
    S.nax[n] = flush(ax);
    S.nay[n] = flush(ay);
}

// ---------------------------------------------------------------------------
// Phase 2 (USF): strain, volume and stress update (scheme.py:31-35 ->
// particle.py:249-327, material.py), external and internal forces
// (scheme.py:37-56 -> element.py:204-303, 842-901) and the nodal update
// (element.py:305-329).
// Phase 2 (USL): forces and nodal update only; the stress update runs after
// G2P (scheme.py:127-133).
// ---------------------------------------------------------------------------
template <bool USL, bool REINIT, bool TRAC>
__global__ void __launch_bounds__(TILE_THREADS)
k_forces(const SimDev* __restrict__ sims, const int4* __restrict__ tiles,
         Control* __restrict__ ctl) {
    __shared__ float s_f[4][4][TILE_THREADS];   // [fint x, fint y, fext x, fext y][corner][cell]
    const int4 T = tiles[blockIdx.x];
    const SimDev& S = sims[T.x];
    const int step = load_step(ctl);
    const int parity = step & 1, next = parity ^ 1;
    const float t = step_time(step, S.dt);
    const int tid = threadIdx.x, lx = tid & (TILE_CX - 1), ly = tid / TILE_CX;
    const int c0x = T.y * TILE_NX - 1, c0y = T.z * TILE_NY - 1;
    const int ci = c0x + lx, cj = c0y + ly;
    const bool owned = lx >= 1 && ly >= 1;

    float fix[4] = {0.f, 0.f, 0.f, 0.f}, fiy[4] = {0.f, 0.f, 0.f, 0.f};
    float fex[4] = {0.f, 0.f, 0.f, 0.f}, fey[4] = {0.f, 0.f, 0.f, 0.f};
    if (ci >= 0 && ci < S.nx && cj >= 0 && cj < S.ny) {
        const CellGeo g = cell_geo(ci, cj, S.hx, S.hy);
        float V0 = 0.0f, size0 = 1.0f;
        if (REINIT) {
            const int cnt = count_cell(S, ci, cj, g);
            if (cnt) V0 = fdv(S.vol_el, (float)cnt);
            size0 = sqrtf(V0);
        }
        float nvx[4], nvy[4], dvol = 0.0f;
        if (!USL) {
            int ids[4];
            cell_nodes(S, ci, cj, ids);
            #pragma unroll
            for (int k = 0; k < 4; ++k) {
                nvx[k] = S.nvax[ids[k]];
                nvy[k] = S.nvay[ids[k]];
            }
            // centroid strain rate (xi = eta = 0), particle.py:270-279
            float Gcx[4], Gcy[4], c0, c1, c3;
            dshape4(0.0f, 0.0f, g.rx, g.ry, Gcx, Gcy);
            strain_rate4(Gcx, Gcy, nvx, nvy, c0, c1, c3);
            dvol = fm(S.dt, fa(c0, c1));
        }
        const float* __restrict__ sxx = S.sxx[parity];
        const float* __restrict__ syy = S.syy[parity];
        const float* __restrict__ szz = S.szz[parity];
        const float* __restrict__ sxy = S.sxy[parity];
        const float* __restrict__ rho = S.rho[parity];
        const float* __restrict__ vsc = S.vsc[parity];
        visit_cell(S, ci, cj, g, [&](int q) {
            const float xi = natural(S.x[q], g.cx, g.rx);
            const float eta = natural(S.y[q], g.cy, g.ry);
            float N[4], Gx[4], Gy[4];
            shape4(xi, eta, N);
            dshape4(xi, eta, g.rx, g.ry, Gx, Gy);
            PState p;
            p.sxx = sxx[q];
            p.syy = syy[q];
            p.szz = szz[q];
            p.sxy = sxy[q];
            p.rho = rho[q];
            const float mp = REINIT ? fm(V0, p.rho) : S.mass[q];
            float V = REINIT ? V0 : S.vol[parity][q];
            if (!USL) {
                float r0, r1, r3;
                strain_rate4(Gx, Gy, nvx, nvy, r0, r1, r3);
                p.exx = S.exx[q];
                p.eyy = S.eyy[q];
                p.exy = S.exy[q];
                p.vsc = vsc[q];
                const MatDev M = S.mats[S.mat[q]];
                const float Ep = S.E ? S.E[q] : -1.0f;
                V = fm(V, strain_stress_update(M, Ep, S.dt, r0, r1, r3, dvol, p));
                if (owned) {
                    S.sxx[next][q] = p.sxx;
                    S.syy[next][q] = p.syy;
                    S.szz[next][q] = p.szz;
                    S.sxy[next][q] = p.sxy;
                    S.exx[q] = p.exx;
                    S.eyy[q] = p.eyy;
                    S.exy[q] = p.exy;
                    S.rho[next][q] = p.rho;
                    S.vsc[next][q] = p.vsc;
                    if (!REINIT) S.vol[next][q] = V;
                }
            }
            // internal force (element.py:868-878)
            const float nV = -V;
            #pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float fx = fa(fm(Gx[k], p.sxx), fm(Gy[k], p.sxy));
                const float fy = fa(fm(Gy[k], p.syy), fm(Gx[k], p.sxy));
                fix[k] = fa(fix[k], fm(nV, fx));
                fiy[k] = fa(fiy[k], fm(nV, fy));
            }
            // body force (element.py:252-256)
            const float mgx = fm(mp, S.gx), mgy = fm(mp, S.gy);
            #pragma unroll
            for (int k = 0; k < 4; ++k) {
                fex[k] = fa(fex[k], fm(N[k], mgx));
                fey[k] = fa(fey[k], fm(N[k], mgy));
            }
            add_traction<TRAC>(S, q, t, V, REINIT ? size0 : (S.psize ? S.psize[q] : 1.0f), N,
                               fex, fey);
        });
    }
    #pragma unroll
    for (int k = 0; k < 4; ++k) {
        s_f[0][k][tid] = fix[k];
        s_f[1][k][tid] = fiy[k];
        s_f[2][k][tid] = fex[k];
        s_f[3][k][tid] = fey[k];
    }
    __syncthreads();
    if (lx < TILE_NX && ly < TILE_NY) {
        const int I = c0x + 1 + lx, J = c0y + 1 + ly;
        if (I <= S.nx && J <= S.ny) {
            nodal_update(S, J * (S.nx + 1) + I, t, node_sum(s_f[0], tid), node_sum(s_f[1], tid),
                         node_sum(s_f[2], tid), node_sum(s_f[3], tid));
        }
    }
}

// ---------------------------------------------------------------------------
// Phase 3: G2P (diffmpm/particle.py:208-247): v_hat = sum N v_i,
// a_hat = sum N a_i, v_p = v_hat or v_p + a_hat dt, x_p += v_hat dt.  USL adds
// the strain/volume/stress update at the step's natural coordinates with the
// updated nodal velocities (scheme.py:127-133).  Thread per owned sort-cell.
// ---------------------------------------------------------------------------
template <bool USL, bool REINIT>
__global__ void __launch_bounds__(TILE_THREADS)
k_particle_kinematics(const SimDev* __restrict__ sims, const int4* __restrict__ tiles,
                      Control* __restrict__ ctl) {
    const int4 T = tiles[blockIdx.x];
    const SimDev& S = sims[T.x];
    const int step = load_step(ctl);
    const int parity = step & 1, next = parity ^ 1;
    const int tid = threadIdx.x, lx = tid & (TILE_CX - 1), ly = tid / TILE_CX;
    int status = 0;
    if (lx < TILE_NX && ly < TILE_NY) {
        const int si = T.y * TILE_NX + lx, sj = T.z * TILE_NY + ly;
        if (si < S.nx && sj < S.ny) {
            const int s = sj * S.nx + si;
            const int b = S.cstart[s], e = S.cstart[s + 1];
            const bool flagged = S.cflag[s] != 0;
            bool drifted = false;
            int cci = -1, ccj = -1;
            CellGeo g;
            float nvx[4], nvy[4], nax[4], nay[4], dvol = 0.0f, V0 = 0.0f;
            const float dt = S.dt;
            #pragma unroll 1
            for (int q = b; q < e; ++q) {
                const float x = S.x[q], y = S.y[q];
                int ci = si, cj = sj;
                if (flagged) {
                    ci = locate_axis(x, S.hx, S.nx);
                    cj = locate_axis(y, S.hy, S.ny);
                    if (ci < 0 || ci >= S.nx || cj < 0 || cj >= S.ny) {
                        status |= ST_OUT_OF_MESH;
                        continue;
                    }
                }
                if (ci != cci || cj != ccj) {
                    cci = ci;
                    ccj = cj;
                    g = cell_geo(ci, cj, S.hx, S.hy);
                    int ids[4];
                    cell_nodes(S, ci, cj, ids);
                    #pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        nvx[k] = S.nvbx[ids[k]];
                        nvy[k] = S.nvby[ids[k]];
                        nax[k] = S.nax[ids[k]];
                        nay[k] = S.nay[ids[k]];
                    }
                    if (USL) {
                        float Gcx[4], Gcy[4], c0, c1, c3;
                        dshape4(0.0f, 0.0f, g.rx, g.ry, Gcx, Gcy);
                        strain_rate4(Gcx, Gcy, nvx, nvy, c0, c1, c3);
                        dvol = fm(dt, fa(c0, c1));
                    }
                }
                const float xi = natural(x, g.cx, g.rx);
                const float eta = natural(y, g.cy, g.ry);
                float N[4];
                shape4(xi, eta, N);
                const float vhx = dot4(N, nvx), vhy = dot4(N, nvy);
                float vx, vy;
                if (S.velocity_update) {
                    vx = vhx;
                    vy = vhy;
                } else {
                    vx = fa(S.vx[q], fm(dot4(N, nax), dt));
                    vy = fa(S.vy[q], fm(dot4(N, nay), dt));
                }
                const float xn = fa(x, fm(vhx, dt)), yn = fa(y, fm(vhy, dt));
                S.x[q] = xn;
                S.y[q] = yn;
                S.vx[q] = vx;
                S.vy[q] = vy;
                if (USL) {
                    float Gx[4], Gy[4], r0, r1, r3;
                    dshape4(xi, eta, g.rx, g.ry, Gx, Gy);
                    strain_rate4(Gx, Gy, nvx, nvy, r0, r1, r3);
                    PState p;
                    p.sxx = S.sxx[parity][q];
                    p.syy = S.syy[parity][q];
                    p.szz = S.szz[parity][q];
                    p.sxy = S.sxy[parity][q];
                    p.exx = S.exx[q];
                    p.eyy = S.eyy[q];
                    p.exy = S.exy[q];
                    p.rho = S.rho[parity][q];
                    p.vsc = S.vsc[parity][q];
                    const MatDev M = S.mats[S.mat[q]];
                    const float Ep = S.E ? S.E[q] : -1.0f;
                    const float f = strain_stress_update(M, Ep, dt, r0, r1, r3, dvol, p);
                    S.sxx[next][q] = p.sxx;
                    S.syy[next][q] = p.syy;
                    S.szz[next][q] = p.szz;
                    S.sxy[next][q] = p.sxy;
                    S.exx[q] = p.exx;
                    S.eyy[q] = p.eyy;
                    S.exy[q] = p.exy;
                    S.rho[next][q] = p.rho;
                    S.vsc[next][q] = p.vsc;
                    if (!REINIT) S.vol[next][q] = fm(S.vol[parity][q], f);
                    (void)V0;
                }
                const int ni = locate_axis(xn, S.hx, S.nx), nj = locate_axis(yn, S.hy, S.ny);
                if (ni < 0 || ni >= S.nx || nj < 0 || nj >= S.ny) {
                    status |= ST_OUT_OF_MESH;
                } else {
                    const int d = max(abs(ni - si), abs(nj - sj));
                    if (d >= 1) drifted = true;
                    if (d > 1) status |= ST_DRIFT_VIOLATION;
                }
            }
            S.cflag[s] = drifted ? 1 : 0;
            if (drifted) status |= ST_DRIFTED;
        }
    }
    // block-wide OR of the status bits, then one atomic per CTA
    status = __reduce_or_sync(0xffffffffu, status);
    __shared__ int s_status;
    if (tid == 0) s_status = 0;
    __syncthreads();
    if ((tid & 31) == 0 && status) atomicOr(&s_status, status);
    __syncthreads();
    if (tid == 0) {
        if (s_status) atomicOr(&ctl->status, s_status);
        // last CTA to finish advances the step counter (every CTA has read it)
        __threadfence();
        const unsigned prev = atomicAdd(&ctl->done, 1u);
        if (prev == gridDim.x - 1) {
            ctl->done = 0u;
            ctl->step = step + 1;
            __threadfence();
        }
    }
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
cudaError_t launch_nodal_kinematics(const StepConfig& c, const SimDev* sims, const int4* tiles,
                                    int ntiles, Control* ctl, cudaStream_t s) {
    if (c.reinit) k_nodal_kinematics<true><<<ntiles, TILE_THREADS, 0, s>>>(sims, tiles, ctl);
    else k_nodal_kinematics<false><<<ntiles, TILE_THREADS, 0, s>>>(sims, tiles, ctl);
    return cudaGetLastError();
}

template <bool USL, bool REINIT>
static void forces_trac(bool trac, const SimDev* sims, const int4* tiles, int ntiles, Control* ctl,
                        cudaStream_t s) {
    if (trac) k_forces<USL, REINIT, true><<<ntiles, TILE_THREADS, 0, s>>>(sims, tiles, ctl);
    else k_forces<USL, REINIT, false><<<ntiles, TILE_THREADS, 0, s>>>(sims, tiles, ctl);
}

cudaError_t launch_forces(const StepConfig& c, const SimDev* sims, const int4* tiles, int ntiles,
                          Control* ctl, cudaStream_t s) {
    if (c.usl) {
        if (c.reinit) forces_trac<true, true>(c.traction, sims, tiles, ntiles, ctl, s);
        else forces_trac<true, false>(c.traction, sims, tiles, ntiles, ctl, s);
    } else {
        if (c.reinit) forces_trac<false, true>(c.traction, sims, tiles, ntiles, ctl, s);
        else forces_trac<false, false>(c.traction, sims, tiles, ntiles, ctl, s);
    }
    return cudaGetLastError();
}

cudaError_t launch_particle_kinematics(const StepConfig& c, const SimDev* sims, const int4* tiles,
                                       int ntiles, Control* ctl, cudaStream_t s) {
    if (c.usl) {
        if (c.reinit) k_particle_kinematics<true, true><<<ntiles, TILE_THREADS, 0, s>>>(sims, tiles, ctl);
        else k_particle_kinematics<true, false><<<ntiles, TILE_THREADS, 0, s>>>(sims, tiles, ctl);
    } else {
        if (c.reinit) k_particle_kinematics<false, true><<<ntiles, TILE_THREADS, 0, s>>>(sims, tiles, ctl);
        else k_particle_kinematics<false, false><<<ntiles, TILE_THREADS, 0, s>>>(sims, tiles, ctl);
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Re-sort: key = current cell (ncell for a particle outside the mesh), counting
// sort with atomic placement, then each bucket sorted by storage index, so the
// result is the stable order whatever the placement order was.
// ---------------------------------------------------------------------------
__global__ void k_resort_keys(const SimDev* __restrict__ sim, int np, int nx, int ny, float hx,
                              float hy, int* __restrict__ count, int* __restrict__ key,
                              Control* __restrict__ ctl) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const int i = locate_axis(sim->x[q], hx, nx);
    const int j = locate_axis(sim->y[q], hy, ny);
    int k;
    if (i < 0 || i >= nx || j < 0 || j >= ny) {
        k = nx * ny;
        atomicOr(&ctl->status, ST_OUT_OF_MESH);
    } else {
        k = j * nx + i;
    }
    key[q] = k;
    atomicAdd(&count[k], 1);
}

cudaError_t launch_resort_keys(const SimDev* sim, int np, int nx, int ny, float hx, float hy,
                               const SortScratch& w, Control* ctl, cudaStream_t s) {
    if (np > 0)
        k_resort_keys<<<(np + 255) / 256, 256, 0, s>>>(sim, np, nx, ny, hx, hy, w.count, w.key, ctl);
    return cudaGetLastError();
}

// exclusive scan, 1024 elements per block
__device__ __forceinline__ int block_exclusive_scan(int v, int* total) {
    __shared__ int warp_sums[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
    #pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int w = (lane < (int)(blockDim.x >> 5)) ? warp_sums[lane] : 0;
        #pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    const int base = wid ? warp_sums[wid - 1] : 0;
    if (total) *total = warp_sums[(blockDim.x >> 5) - 1];
    __syncthreads();
    return base + x - v;
}

__global__ void k_scan_blocks(const int* __restrict__ in, int* __restrict__ out, int n,
                              int* __restrict__ block_sums) {
    const int i = blockIdx.x * 1024 + threadIdx.x;
    const int v = i < n ? in[i] : 0;
    int total;
    const int ex = block_exclusive_scan(v, &total);
    if (i < n) out[i] = ex;
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

__global__ void k_scan_sums(int* __restrict__ block_sums, int nb) {
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += 1024) {
        const int i = base + threadIdx.x;
        const int v = i < nb ? block_sums[i] : 0;
        int total;
        const int ex = block_exclusive_scan(v, &total);
        if (i < nb) block_sums[i] = ex + carry;
        __syncthreads();
        if (threadIdx.x == 0) carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) block_sums[nb] = carry;
}

__global__ void k_scan_add(int* __restrict__ out, int n, const int* __restrict__ block_sums) {
    const int i = blockIdx.x * 1024 + threadIdx.x;
    if (i < n) out[i] += block_sums[blockIdx.x];
    if (i == n) out[n] = block_sums[gridDim.x];   // grand total
}

cudaError_t launch_exclusive_scan(const int* in, int* out, int n, int* block_sums,
                                  cudaStream_t s) {
    const int nb = (n + 1024) / 1024;   // room for out[n]
    k_scan_blocks<<<nb, 1024, 0, s>>>(in, out, n, block_sums);
    k_scan_sums<<<1, 1024, 0, s>>>(block_sums, nb);
    k_scan_add<<<nb, 1024, 0, s>>>(out, n, block_sums);
    return cudaGetLastError();
}

__global__ void k_resort_place(int np, const int* __restrict__ start, const int* __restrict__ key,
                               int* __restrict__ cursor, int* __restrict__ perm) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= np) return;
    const int k = key[q];
    perm[start[k] + atomicAdd(&cursor[k], 1)] = q;
}

cudaError_t launch_resort_place(int np, const int* start, const SortScratch& w, cudaStream_t s) {
    if (np > 0) k_resort_place<<<(np + 255) / 256, 256, 0, s>>>(np, start, w.key, w.cursor, w.perm);
    return cudaGetLastError();
}

__global__ void k_resort_segsort(int nbucket, const int* __restrict__ start,
                                 int* __restrict__ perm) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nbucket) return;
    const int b = start[c], e = start[c + 1];
    #pragma unroll 1
    for (int i = b + 1; i < e; ++i) {
        const int v = perm[i];
        int j = i - 1;
        #pragma unroll 1
        while (j >= b && perm[j] > v) {
            perm[j + 1] = perm[j];
            --j;
        }
        perm[j + 1] = v;
    }
}

cudaError_t launch_resort_segsort(int nbucket, const int* start, const SortScratch& w,
                                  cudaStream_t s) {
    if (nbucket > 0) k_resort_segsort<<<(nbucket + 255) / 256, 256, 0, s>>>(nbucket, start, w.perm);
    return cudaGetLastError();
}

template <class T>
__global__ void k_gather(const T* __restrict__ src, T* __restrict__ dst,
                         const int* __restrict__ perm, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[perm[i]];
}

template <class T>
__global__ void k_gather_pair(const T* __restrict__ src, T* __restrict__ dst,
                              const int* __restrict__ perm, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const int p = perm[i];
        dst[2 * i] = src[2 * p];
        dst[2 * i + 1] = src[2 * p + 1];
    }
}

cudaError_t launch_gather_u32(const uint32_t* src, uint32_t* dst, const int* perm, int n,
                              cudaStream_t s) {
    if (n > 0) k_gather<uint32_t><<<(n + 255) / 256, 256, 0, s>>>(src, dst, perm, n);
    return cudaGetLastError();
}
cudaError_t launch_gather_u8(const uint8_t* src, uint8_t* dst, const int* perm, int n,
                             cudaStream_t s) {
    if (n > 0) k_gather<uint8_t><<<(n + 255) / 256, 256, 0, s>>>(src, dst, perm, n);
    return cudaGetLastError();
}
cudaError_t launch_gather_pair_u32(const uint32_t* src, uint32_t* dst, const int* perm, int n,
                                   cudaStream_t s) {
    if (n > 0) k_gather_pair<uint32_t><<<(n + 255) / 256, 256, 0, s>>>(src, dst, perm, n);
    return cudaGetLastError();
}
cudaError_t launch_gather_pair_u8(const uint8_t* src, uint8_t* dst, const int* perm, int n,
                                  cudaStream_t s) {
    if (n > 0) k_gather_pair<uint8_t><<<(n + 255) / 256, 256, 0, s>>>(src, dst, perm, n);
    return cudaGetLastError();
}

// Volume set-up of a freshly sorted population (particle.py:158-178):
// V = V_el / count, size = sqrt(V), m = V rho.
__global__ void k_setup_volume(const SimDev* __restrict__ sim, int np, int parity) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const SimDev& S = *sim;
    if (q >= np) return;
    const int i = locate_axis(S.x[q], S.hx, S.nx), j = locate_axis(S.y[q], S.hy, S.ny);
    if (i < 0 || i >= S.nx || j < 0 || j >= S.ny) return;
    const int c = j * S.nx + i;
    const int cnt = S.cstart[c + 1] - S.cstart[c];
    const float V = fdv(S.vol_el, (float)cnt);
    S.vol[parity][q] = V;
    S.mass[q] = fm(V, S.rho[parity][q]);
    if (S.psize) S.psize[q] = sqrtf(V);
}

cudaError_t launch_setup_volume(const SimDev* sim, int np, int parity, cudaStream_t s) {
    if (np > 0) k_setup_volume<<<(np + 255) / 256, 256, 0, s>>>(sim, np, parity);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Field transfers
// ---------------------------------------------------------------------------
__global__ void k_scatter_out(const float* const* __restrict__ comp, int ncomp,
                              const int* __restrict__ pid, int np, float* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const int o = pid[i];
    for (int c = 0; c < ncomp; ++c) out[(size_t)o * ncomp + c] = comp[c] ? comp[c][i] : 0.0f;
}

cudaError_t launch_scatter_out(const float* const* comp_ptrs, int ncomp, const int* pid, int np,
                               float* out, cudaStream_t s) {
    if (np > 0) k_scatter_out<<<(np + 255) / 256, 256, 0, s>>>(comp_ptrs, ncomp, pid, np, out);
    return cudaGetLastError();
}

__global__ void k_gather_in(float* const* __restrict__ comp, int ncomp,
                            const int* __restrict__ pid, int np, const float* __restrict__ in) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const int o = pid[i];
    for (int c = 0; c < ncomp; ++c)
        if (comp[c]) comp[c][i] = in[(size_t)o * ncomp + c];
}

cudaError_t launch_gather_in(float* const* comp_ptrs, int ncomp, const int* pid, int np,
                             const float* in, cudaStream_t s) {
    if (np > 0) k_gather_in<<<(np + 255) / 256, 256, 0, s>>>(comp_ptrs, ncomp, pid, np, in);
    return cudaGetLastError();
}

__global__ void k_gather_in_u8(uint8_t* __restrict__ dst, const int* __restrict__ pid, int np,
                               const int32_t* __restrict__ in) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < np) dst[i] = (uint8_t)in[pid[i]];
}

cudaError_t launch_gather_in_u8(uint8_t* dst, const int* pid, int np, const int32_t* in,
                                cudaStream_t s) {
    if (np > 0) k_gather_in_u8<<<(np + 255) / 256, 256, 0, s>>>(dst, pid, np, in);
    return cudaGetLastError();
}

__global__ void k_scatter_out_u8(const uint8_t* __restrict__ src, const int* __restrict__ pid,
                                 int np, int32_t* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < np) out[pid[i]] = src[i];
}

cudaError_t launch_scatter_out_u8(const uint8_t* src, const int* pid, int np, int32_t* out,
                                  cudaStream_t s) {
    if (np > 0) k_scatter_out_u8<<<(np + 255) / 256, 256, 0, s>>>(src, pid, np, out);
    return cudaGetLastError();
}

// what: 0 element id (int32), 1 volume, 2 mass, 3 momentum (2 comps)
__global__ void k_derived_out(const SimDev* __restrict__ sim, int np, int parity, int reinit,
                              int what, const int* __restrict__ pid, void* __restrict__ out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const SimDev& S = *sim;
    if (q >= np) return;
    const int o = pid[q];
    const int i = locate_axis(S.x[q], S.hx, S.nx), j = locate_axis(S.y[q], S.hy, S.ny);
    const bool in = i >= 0 && i < S.nx && j >= 0 && j < S.ny;
    float V, m;
    if (reinit) {
        // the volume set-up at the current positions (the cells are sorted)
        int cnt = 0;
        if (in) {
            const int c = j * S.nx + i;
            cnt = S.cstart[c + 1] - S.cstart[c];
        }
        V = cnt ? fdv(S.vol_el, (float)cnt) : 0.0f;
        m = fm(V, S.rho[parity][q]);
    } else {
        V = S.vol[parity][q];
        m = S.mass[q];
    }
    if (what == 0) {
        static_cast<int32_t*>(out)[o] = in ? j * S.nx + i : -1;
    } else if (what == 1) {
        static_cast<float*>(out)[o] = V;
    } else if (what == 2) {
        static_cast<float*>(out)[o] = m;
    } else {
        static_cast<float*>(out)[2 * (size_t)o] = fm(m, S.vx[q]);
        static_cast<float*>(out)[2 * (size_t)o + 1] = fm(m, S.vy[q]);
    }
}

cudaError_t launch_derived_out(const SimDev* sim, int np, int parity, bool reinit, int what,
                               const int* pid, void* out, cudaStream_t s) {
    if (np > 0)
        k_derived_out<<<(np + 255) / 256, 256, 0, s>>>(sim, np, parity, reinit ? 1 : 0, what, pid, out);
    return cudaGetLastError();
}

__global__ void k_interleave2(const float* __restrict__ a, const float* __restrict__ b, int n,
                              float* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        out[2 * i] = a[i];
        out[2 * i + 1] = b[i];
    }
}
__global__ void k_deinterleave2(const float* __restrict__ in, int n, float* __restrict__ a,
                                float* __restrict__ b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        a[i] = in[2 * i];
        b[i] = in[2 * i + 1];
    }
}
__global__ void k_node_momentum(const float* __restrict__ m, const float* __restrict__ vx,
                                const float* __restrict__ vy, int n, float* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        out[2 * i] = fm(m[i], vx[i]);
        out[2 * i + 1] = fm(m[i], vy[i]);
    }
}

cudaError_t launch_interleave2(const float* a, const float* b, int n, float* out, cudaStream_t s) {
    if (n > 0) k_interleave2<<<(n + 255) / 256, 256, 0, s>>>(a, b, n, out);
    return cudaGetLastError();
}
cudaError_t launch_deinterleave2(const float* in, int n, float* a, float* b, cudaStream_t s) {
    if (n > 0) k_deinterleave2<<<(n + 255) / 256, 256, 0, s>>>(in, n, a, b);
    return cudaGetLastError();
}
cudaError_t launch_node_momentum(const float* m, const float* vx, const float* vy, int n,
                                 float* out, cudaStream_t s) {
    if (n > 0) k_node_momentum<<<(n + 255) / 256, 256, 0, s>>>(m, vx, vy, n, out);
    return cudaGetLastError();
}

}  // namespace mpm
