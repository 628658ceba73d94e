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
#include <cstddef>
#include <cstdint>
#include <type_traits>
#include "mpm_device.cuh"
#include "mpm_kernels.h"

namespace mpm {

__device__ __forceinline__ int load_step(const Control* ctl) {
    return *reinterpret_cast<const volatile int*>(&ctl->step);
}

// Batched launches: per step block, every tile gets a record with its
// simulation's descriptor and control pointer, the storage starts of its
// cell rows and its occupancy (one warp per record).
__global__ void k_gather_tiles(const SimDev* const* __restrict__ sims, Control* const* __restrict__ ctls,
                               const int4* __restrict__ tiles, int ntiles, TileDesc* __restrict__ out) {
    const int t = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31;
    if (t >= ntiles) return;
    const int4 T = tiles[t];
    TileDesc& d = out[t];
    if (T.x < 0) {   // past the end of a classified list
        if (lane == 0) d.T = T;
        return;
    }
    if (lane == 0) {
        d.T = T;
        d.ctl = ctls[T.x];
        d.pad = 0;
    }
    const SimDev* sd = sims[T.x];
    const int* a = reinterpret_cast<const int*>(sd);
    int* b = reinterpret_cast<int*>(&d.S);
    for (int i = lane; i < (int)(sizeof(SimDev) / 4); i += 32) b[i] = a[i];
    const int nx = sd->nx, ny = sd->ny;
    const int* __restrict__ cstart = sd->cstart;
    const int c0x = T.y * TILE_NX - 1, c0y = T.z * TILE_NY - 1;
    #pragma unroll 1
    for (int r = 0; r < TILE_CY; ++r) {
        const int cj = c0y + r;
        const bool in = cj >= 0 && cj < ny;
        d.cs[r][lane] = in ? cstart[cj * nx + min(max(c0x + lane, 0), nx)] : 0;
        if (lane == 0) d.cs[r][32] = in ? cstart[cj * nx + min(max(c0x + 32, 0), nx)] : 0;
    }
    int occ = 0;
    const int x0 = max(c0x - 1, 0), x1 = min(c0x + TILE_CX + 1, nx);
    const int y0 = max(c0y - 1, 0), y1 = min(c0y + TILE_CY + 1, ny);
    if (x0 < x1)
        for (int r = y0 + lane; r < y1; r += 32) occ |= cstart[r * nx + x1] != cstart[r * nx + x0];
    occ = __any_sync(0xffffffffu, occ);
    if (lane == 0) {
        d.occ = occ;
        d.pad2[0] = d.pad2[1] = d.pad2[2] = 0;
    }
}

cudaError_t launch_gather_tiles(const SimDev* const* sims, Control* const* ctls, const int4* tiles,
                                int ntiles, TileDesc* out, cudaStream_t s) {
    if (ntiles > 0) k_gather_tiles<<<(ntiles + 7) / 8, 256, 0, s>>>(sims, ctls, tiles, ntiles, out);
    return cudaGetLastError();
}

// A batched CTA copies its tile record (tile, control pointer, descriptor,
// row starts) into shared memory, 16 bytes per thread.
__device__ __forceinline__ void load_tile(const TileDesc* __restrict__ src, TileDesc& dst) {
    const int4* a = reinterpret_cast<const int4*>(src);
    int4* b = reinterpret_cast<int4*>(&dst);
    for (int i = threadIdx.x; i < (int)(sizeof(TileDesc) / 16); i += blockDim.x) b[i] = a[i];
    __syncthreads();
}

// The step counter advances once per launch sequence, after its last kernel:
// the step kernels read step = counter + k (k their offset in the sequence).
__global__ void k_advance_steps(Control* const* __restrict__ ctls, Control* __restrict__ one, int n,
                                int by) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (one) {
        if (i == 0) one->step += by;
    } else if (i < n) {
        ctls[i]->step += by;
    }
}

cudaError_t launch_advance_steps(Control* const* ctls, int n, int by, cudaStream_t s) {
    if (n > 0 && by != 0) k_advance_steps<<<(n + 127) / 128, 128, 0, s>>>(ctls, nullptr, n, by);
    return cudaGetLastError();
}

cudaError_t launch_advance_step(Control* ctl, int by, cudaStream_t s) {
    if (by != 0) k_advance_steps<<<1, 32, 0, s>>>(nullptr, ctl, 1, by);
    return cudaGetLastError();
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

// A descriptor field read at its point of use.  With VD (the descriptor is a
// shared-memory copy, batched kernels) the read is volatile, so the compiler
// reloads the field instead of keeping ~20 loop-invariant pointers live in
// registers (which spilled); a __grid_constant__ descriptor is read from the
// constant bank either way.
template <bool VD, class T>
__device__ __forceinline__ T rd(const T& f) {
    if constexpr (VD) return *const_cast<const volatile T*>(&f);
    else return f;
}


template <bool VD = false>
__device__ __forceinline__ void apply_constraint(const SimDev& S, uint16_t code, float& vx,
                                                 float& vy, float* ax, float* ay) {
    const int c0 = code & 0xff, c1 = code >> 8;
    if (c0) {
        vx = rd<VD>(S.cons_vel)[c0 - 1];
        if (ax) *ax = 0.0f;
    }
    if (c1) {
        vy = rd<VD>(S.cons_vel)[c1 - 1];
        if (ay) *ay = 0.0f;
    }
}

// ---------------------------------------------------------------------------
// Tile streaming.
//
// Fast path (no drift flag set on the 34 x 18 sort-cells around the tile, so
// every particle of the tile is in its sort-cell): warp w streams the
// contiguous storage range of cell row w in chunks of 32 particles, one
// particle per lane.  The chunks are staged into shared memory with cp.async
// copies issued several chunks ahead, so a warp keeps DEPTH-1 chunks of loads
// in flight while it computes.  A particle's cell is found from its storage
// index by a binary search of the row's cell starts, and the cell geometry
// comes from per-tile tables, so no division or locate runs per particle.  The
// particle's NQ corner contributions go to shared-memory slots; lane l then
// adds, in storage order, the slots of the particles of its own cell
// (c0x + l, row w) to that cell's partials.
// Slow path (some neighbouring particle drifted): each thread visits the
// particles currently in its cell with visit_cell.  Both paths use the same
// per-particle function and the same per-cell values and add in the same order
// (storage order within the cell), so on an undrifted tile they give bitwise
// the same partials.
// ---------------------------------------------------------------------------
constexpr int HALO_W = TILE_CX + 2;   // sort-cells checked for drift: [c0x-1, c0x+33)
constexpr int HALO_H = TILE_CY + 2;   //                               [c0y-1, c0y+17)
constexpr int GEO_C = TILE_CX + 3;    // geometry table columns k <-> cell c0x - 1 + k
constexpr int GEO_R = TILE_CY + 3;    // geometry table rows    k <-> cell c0y - 1 + k

// Per-tile cell geometry: bounds, centre and 2/width of columns and rows, formed
// exactly as cell_geo forms them, one 16-byte entry per column and per row.
struct TileGeo {
    float4 col[GEO_C];   // (x0, x1, cx, rx) of cell column c0x - 1 + k
    float4 row[GEO_R];   // (y0, y1, cy, ry) of cell row    c0y - 1 + k
};

__device__ __forceinline__ float4 axis_geo(int i, float h) {
    const float a = node_coord(i, h), b = node_coord(i + 1, h);
    return make_float4(a, b, fm(fa(a, b), 0.5f), fdv(2.0f, fs(b, a)));
}

__device__ __forceinline__ void build_geo(const SimDev& S, int c0x, int c0y, TileGeo& G) {
    const int t = threadIdx.x;
    if (t < GEO_C) G.col[t] = axis_geo(c0x - 1 + t, S.hx);
    else if (t >= 64 && t < 64 + GEO_R) G.row[t - 64] = axis_geo(c0y - 1 + (t - 64), S.hy);
}

__device__ __forceinline__ CellGeo geo_of(const TileGeo& G, int kc, int kr) {
    const float4 c = G.col[kc], r = G.row[kr];
    CellGeo g;
    g.x0 = c.x;
    g.x1 = c.y;
    g.cx = c.z;
    g.rx = c.w;
    g.y0 = r.x;
    g.y1 = r.y;
    g.cy = r.z;
    g.ry = r.w;
    return g;
}


// The cell l in [0, last] whose range [cs[l], cs[l+1]) holds storage index q
// (the last l with cs[l] <= q; q lies in [cs[0], cs[last+1])).
__device__ __forceinline__ int cell_of(const int* cs, int last, int q) {
    int lo = 0, hi = last;
    #pragma unroll 1
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (cs[mid] <= q) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// The tile set-up loads, all issued before any is consumed so that they cost
// one round trip: the storage starts of the tile's cell row cj (lane l: column
// c0x + l, lane 0 also column c0x + 32), whether a particle is stored in the
// sort-cells [c0x-1, c0x+33) x [c0y-1, c0y+17) (a particle is at most one
// cell from its sort-cell, so when the cells of a tile and the ring of cells
// around them store no particle, no particle is in the tile's cells), and
// whether any of them has its drift flag set (the tile then takes the
// gathering path).
struct TileLoads {
    int cs, cs32;     // row starts
    int occ, drift;   // this thread's share of the two block-wide ORs
};

// The drift-flag share of tile_loads.
__device__ __forceinline__ int tile_drift(const SimDev& S, int c0x, int c0y) {
    int drift = 0;
    for (int idx = threadIdx.x; idx < HALO_W * HALO_H; idx += TILE_THREADS) {
        const int si = c0x - 1 + idx % HALO_W, sj = c0y - 1 + idx / HALO_W;
        if (si >= 0 && si < S.nx && sj >= 0 && sj < S.ny) drift |= S.cflag[sj * S.nx + si];
    }
    return drift;
}

// tile_loads for a batched tile: the row starts and the occupancy come from
// its record (rec, in shared memory); only the drift flags are loaded.
__device__ __forceinline__ TileLoads record_loads(const SimDev& S, const TileDesc& rec, int c0x, int c0y,
                                                  int r, int lane) {
    TileLoads L;
    L.cs = rec.cs[r][lane];
    L.cs32 = lane == 0 ? rec.cs[r][32] : 0;
    L.occ = rec.occ;
    L.drift = rec.occ ? tile_drift(S, c0x, c0y) : 0;   // an empty tile needs no drift flags
    return L;
}

__device__ __forceinline__ TileLoads tile_loads(const SimDev& S, int c0x, int c0y, int cj, int lane) {
    TileLoads L{0, 0, 0, 0};
    if (cj >= 0 && cj < S.ny) {
        const int base = cj * S.nx;
        L.cs = S.cstart[base + min(max(c0x + lane, 0), S.nx)];
        if (lane == 0) L.cs32 = S.cstart[base + min(max(c0x + 32, 0), S.nx)];
    }
    const int x0 = max(c0x - 1, 0), x1 = min(c0x + TILE_CX + 1, S.nx);
    const int y0 = max(c0y - 1, 0), y1 = min(c0y + TILE_CY + 1, S.ny);
    if (x0 < x1)
        for (int r = y0 + (int)threadIdx.x; r < y1; r += TILE_THREADS)
            L.occ |= S.cstart[r * S.nx + x1] != S.cstart[r * S.nx + x0];
    for (int idx = threadIdx.x; idx < HALO_W * HALO_H; idx += TILE_THREADS) {
        const int si = c0x - 1 + idx % HALO_W, sj = c0y - 1 + idx / HALO_W;
        if (si >= 0 && si < S.nx && sj >= 0 && sj < S.ny) L.drift |= S.cflag[sj * S.nx + si];
    }
    return L;
}

// Per-warp staging of the chunks of a row: chunk c of [rb, re) holds storage
// indices rb + 32c + lane; field f of it lands in buf[c % DEPTH][f][lane].
template <int NF, int DEPTH>
struct RowStage {
    float (*buf)[NF][32];
    const float* src[NF];
    int rb, re, nch, lane;

    __device__ __forceinline__ void issue(int c) {
        const int q = rb + 32 * c + lane;
        if (c < nch && q < re) {
            #pragma unroll
            for (int f = 0; f < NF; ++f)
                if (src[f]) cp_async4(&buf[c % DEPTH][f][lane], src[f] + q);
        }
        cp_async_commit();
    }
    __device__ __forceinline__ void prime() {
        #pragma unroll
        for (int c = 0; c < DEPTH - 1; ++c) issue(c);
    }
    // Issue chunk c + DEPTH - 1 and wait until chunk c has landed.
    __device__ __forceinline__ const float (*advance(int c))[32] {
        issue(c + DEPTH - 1);
        cp_async_wait<DEPTH - 1>();
        return buf[c % DEPTH];
    }
};

// Per-particle contributions of phase 1 to the 4 corners of its cell:
// [m N_k, N_k (m vx), N_k (m vy)] (element.py:138-152, 170-189).  `m` is the
// particle mass (V0 rho under the per-step volume set-up).
__device__ __forceinline__ void mass_contrib(float x, float y, float vx, float vy, float m,
                                             float cx, float rx, float cy, float ry, float* c) {
    const float xi = natural(x, cx, rx);
    const float eta = natural(y, cy, ry);
    float N[4];
    shape4(xi, eta, N);
    const float pvx = fm(m, vx), pvy = fm(m, vy);
    #pragma unroll
    for (int k = 0; k < 4; ++k) {
        c[k] = fm(m, N[k]);
        c[4 + k] = fm(N[k], pvx);
        c[8 + k] = fm(N[k], pvy);
    }
}

// Particle traction t_p[d] = f(t) tau_d V / size (diffmpm/mesh.py:60-77,
// particle.py:329-343), added to the external-force contributions.
template <bool TRAC>
__device__ __forceinline__ void add_traction(const SimDev& S, int q, float t, float V, float size,
                                             const float N[4], float* cex, float* cey) {
    if constexpr (TRAC) {
        #pragma unroll
        for (int d = 0; d < 2; ++d) {
            const int code = S.tr_fn[2 * q + d];
            if (!code) continue;
            const float tv = fm(fn_value(S, code, t), S.tr_tau[2 * q + d]);
            const float tr = fdv(fm(tv, V), size);
            #pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (d == 0) cex[k] = fa(cex[k], fm(N[k], tr));
                else cey[k] = fa(cey[k], fm(N[k], tr));
            }
        }
    }
}

// Per-cell values of phase 2: the volume set-up V0 = V_el / count and
// size0 = sqrt(V0) (particle.py:169-178), and (USF) dt times the centroid
// volumetric strain rate from the cell's nodal velocities (particle.py:270-279).
template <bool USL, bool REINIT, bool VD = false, bool TRAC = true>
__device__ __forceinline__ void force_cell_values(const SimDev& S, int cnt, const CellGeo& g,
                                                  const float nvx[4], const float nvy[4],
                                                  float& V0, float& size0, float& dvol) {
    V0 = 0.0f;
    size0 = 1.0f;
    if (REINIT) {
        if (cnt) V0 = fdv(rd<VD>(S.vol_el), (float)cnt);
        if (TRAC) size0 = sqrtf(V0);   // only particle tractions use the size
    }
    dvol = 0.0f;
    if (!USL) {
        float Gcx[4], Gcy[4], c0, c1, c3;
        dshape4(0.0f, 0.0f, g.rx, g.ry, Gcx, Gcy);
        strain_rate4(Gcx, Gcy, nvx, nvy, c0, c1, c3);
        dvol = fm(rd<VD>(S.dt), fa(c0, c1));
    }
}

// Staged inputs of one particle in phase 2.
struct ForceIn {
    float x, y, sxx, syy, szz, sxy, rho, vol;
};

enum ForceField { FF_X, FF_Y, FF_SXX, FF_SYY, FF_SZZ, FF_SXY, FF_RHO, FF_VOL, FF_N };

template <bool VD = false>
__device__ __forceinline__ ForceIn force_in_global(const SimDev& S, int q, int parity,
                                                   bool reinit) {
    ForceIn in;
    in.x = rd<VD>(S.x)[q];
    in.y = rd<VD>(S.y)[q];
    in.sxx = rd<VD>(S.sxx[parity])[q];
    in.syy = rd<VD>(S.syy[parity])[q];
    in.szz = rd<VD>(S.szz[parity])[q];
    in.sxy = rd<VD>(S.sxy[parity])[q];
    in.rho = rd<VD>(S.rho[parity])[q];
    in.vol = reinit ? 0.0f : rd<VD>(S.vol[parity])[q];
    return in;
}

// The material table of the CTA's simulation, staged in shared memory at
// tile set-up when it has at most MAT_SHARED entries: the stress updates read
// a particle's material there (with one material, without loading the
// particle's material id).
constexpr int MAT_SHARED = 8;
__shared__ MatDev s_mats[MAT_SHARED];

template <bool VD>
__device__ __forceinline__ void stage_materials(const SimDev& S) {
    constexpr int W = (int)(sizeof(MatDev) / 4);
    static_assert(W * 4 == (int)sizeof(MatDev), "material entries are whole words");
    const int n = min(rd<VD>(S.nmat), MAT_SHARED);
    const int* src = reinterpret_cast<const int*>(rd<VD>(S.mats));
    int* dst = reinterpret_cast<int*>(s_mats);
    for (int i = threadIdx.x; i < n * W; i += blockDim.x) dst[i] = src[i];
}

template <bool VD>
__device__ __forceinline__ const MatDev& material_of(const SimDev& S, int q) {
    const int n = rd<VD>(S.nmat);
    if (n == 1) return s_mats[0];
    const int m = rd<VD>(S.mat)[q];
    return n <= MAT_SHARED ? s_mats[m] : rd<VD>(S.mats)[m];
}

// Per-particle work of phase 2 on a particle state held in registers: the
// USF strain/volume/stress update of `p` and `V` (the particle's volume
// before the step; element.py:236-303, 842-901 via particle.py:249-327) and
// the total-force contributions [f x, f y] x 4 corners, internal plus
// external force.  Returns the volume the forces use (the updated one under
// USF).
template <bool USL, bool REINIT, bool TRAC, bool VD = false>
__device__ __forceinline__ float force_core(const SimDev& S, int q, float x, float y, PState& p, float V,
                                            float cx, float rx, float cy, float ry, float size0,
                                            const float nvx[4], const float nvy[4], float dvol,
                                            float t, float* c) {
    const float xi = natural(x, cx, rx);
    const float eta = natural(y, cy, ry);
    float N[4], Gx[4], Gy[4];
    shape4(xi, eta, N);
    dshape4(xi, eta, rx, ry, Gx, Gy);
    const float mp = REINIT ? fm(V, p.rho) : rd<VD>(S.mass)[q];
    if (!USL) {
        float r0, r1, r3;
        strain_rate4(Gx, Gy, nvx, nvy, r0, r1, r3);
        const MatDev& M = material_of<VD>(S, q);
        const float* E = rd<VD>(S.E);
        const float Ep = E ? E[q] : -1.0f;
        V = fm(V, strain_stress_update(M, Ep, rd<VD>(S.dt), r0, r1, r3, dvol, p));
    }
    const float nV = -V;
    const float mgx = fm(mp, rd<VD>(S.gx)), mgy = fm(mp, rd<VD>(S.gy));
    #pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float fx = fa(fm(Gx[k], p.sxx), fm(Gy[k], p.sxy));
        const float fy = fa(fm(Gy[k], p.syy), fm(Gx[k], p.sxy));
        c[k] = fa(fm(nV, fx), fm(N[k], mgx));
        c[4 + k] = fa(fm(nV, fy), fm(N[k], mgy));
    }
    add_traction<TRAC>(S, q, t, V, REINIT ? size0 : (S.psize ? S.psize[q] : 1.0f), N, c, c + 4);
    return V;
}

// The USF state of particle q after the stress update (buffers `next`).
template <bool REINIT, bool VD>
__device__ __forceinline__ void store_state(const SimDev& S, int q, const PState& p, float V, int next) {
    rd<VD>(S.sxx[next])[q] = p.sxx;
    rd<VD>(S.syy[next])[q] = p.syy;
    rd<VD>(S.szz[next])[q] = p.szz;
    rd<VD>(S.sxy[next])[q] = p.sxy;
    rd<VD>(S.exx)[q] = p.exx;
    rd<VD>(S.eyy)[q] = p.eyy;
    rd<VD>(S.exy)[q] = p.exy;
    rd<VD>(S.rho[next])[q] = p.rho;
    rd<VD>(S.vsc[next])[q] = p.vsc;
    if (!REINIT) rd<VD>(S.vol[next])[q] = V;
}

// force_core on a particle read from global memory; the updated state is
// written back when `write` (the particle's cell is owned by the tile).
template <bool USL, bool REINIT, bool TRAC, bool VD = false>
__device__ __forceinline__ void force_contrib(const SimDev& S, int q, const ForceIn& in, float cx,
                                              float rx, float cy, float ry, float V0, float size0,
                                              const float nvx[4], const float nvy[4], float dvol,
                                              int parity, float t, bool write, float* c) {
    const int next = parity ^ 1;
    PState p;
    if (!USL) {
        // state updated but not needed for the forces: loaded early, used late
        p.exx = rd<VD>(S.exx)[q];
        p.eyy = rd<VD>(S.eyy)[q];
        p.exy = rd<VD>(S.exy)[q];
        p.vsc = rd<VD>(S.vsc[parity])[q];
    }
    p.sxx = in.sxx;
    p.syy = in.syy;
    p.szz = in.szz;
    p.sxy = in.sxy;
    p.rho = in.rho;
    const float V = force_core<USL, REINIT, TRAC, VD>(S, q, in.x, in.y, p, REINIT ? V0 : in.vol, cx, rx,
                                                      cy, ry, size0, nvx, nvy, dvol, t, c);
    if (!USL && write) store_state<REINIT, VD>(S, q, p, V, next);
}

// ---------------------------------------------------------------------------
// Phase 1: nodal kinematics (diffmpm/scheme.py:22-29) with the step's volume
// set-up (diffmpm/solver.py:81-85 via tree_unflatten, solver.py:100-111).
//   P2G of mass and momentum (element.py:122-189), nodal velocity
//   (element.py:191-202), velocity constraints (element.py:331-334).
// ---------------------------------------------------------------------------
constexpr int K1_NF = 5;   // x, y, vx, vy, rho (solve_jit) or mass (solve)
// storage slots of a row per pass: a row of 4 particles in each of 32 cells,
// starting anywhere in a 16-byte piece, fits one pass (three CTAs per SM)
constexpr int K1_ROW_P = 132;

template <bool REINIT, bool REC = false>
__device__ __forceinline__ void nodal_kinematics_tile(const SimDev& S, const int4 T,
                                                      Control* __restrict__ ctl, int k,
                                                      const TileDesc* rec = nullptr) {
    constexpr int NQ = 12;
    __shared__ float s_c[NQ][SC_STRIDE];               // [m, px, py] x corner, per cell
    __shared__ __align__(16) float s_row[TILE_CY][K1_NF][K1_ROW_P];  // staged particles of each cell row
    __shared__ int s_cs[TILE_CY][33];
    __shared__ TileGeo G;
    const int parity = (load_step(ctl) + k) & 1;
    const int tid = threadIdx.x, lx = tid & (TILE_CX - 1), ly = tid / TILE_CX;
    const int c0x = T.y * TILE_NX - 1, c0y = T.z * TILE_NY - 1;
    const int ci = c0x + lx, cj = c0y + ly;
    const float* __restrict__ rho = S.rho[parity];
    const bool node_ok = lx < TILE_NX && ly < TILE_NY && c0x + 1 + lx <= S.nx && c0y + 1 + ly <= S.ny;
    const int node = (c0y + 1 + ly) * (S.nx + 1) + c0x + 1 + lx;
    const uint16_t ncons = node_ok ? S.ncons[node] : 0;   // node-phase input, fetched early
    const TileLoads L = REC ? record_loads(S, *rec, c0x, c0y, ly, lx) : tile_loads(S, c0x, c0y, cj, lx);
    if (!__syncthreads_or(L.occ)) {
        // no particle in the tile: every node is massless and keeps its
        // velocity (the node phase below with all sums zero)
        if (node_ok) {
            float vx = flush(S.nvbx[node]), vy = flush(S.nvby[node]);
            apply_constraint(S, ncons, vx, vy, nullptr, nullptr);
            S.nm[node] = 0.0f;
            S.nvax[node] = vx;
            S.nvay[node] = vy;
        }
        return;
    }
    build_geo(S, c0x, c0y, G);
    #pragma unroll
    for (int q = 0; q < NQ; ++q) s_c[q][tid] = 0.0f;
    s_cs[ly][lx] = L.cs;
    if (lx == 0) s_cs[ly][32] = L.cs32;
    const bool slow = __syncthreads_or(L.drift) != 0;

    if (!slow) {
        const int* cs = s_cs[ly];
        const int cb = cs[lx], ce = cs[lx + 1];
        const CellGeo g = geo_of(G, lx + 1, ly + 1);
        const float V0 = (REINIT && ce > cb) ? fdv(S.vol_el, (float)(ce - cb)) : 0.0f;
        float acc[NQ];
        #pragma unroll
        for (int k = 0; k < NQ; ++k) acc[k] = 0.0f;
        const float* const src[K1_NF] = {S.x, S.y, S.vx, S.vy, REINIT ? rho : S.mass};
        float (*buf)[K1_ROW_P] = s_row[ly];
        row_pass16<K1_NF, K1_ROW_P>(buf, src, cs[0], cs[32], cb, ce, lx, [&](int, int j) {
            const float m = REINIT ? fm(V0, buf[4][j]) : buf[4][j];
            float cc[NQ];
            mass_contrib(buf[0][j], buf[1][j], buf[2][j], buf[3][j], m, g.cx, g.rx, g.cy, g.ry, cc);
            #pragma unroll
            for (int k = 0; k < NQ; ++k) acc[k] = fa(acc[k], cc[k]);
        });
        #pragma unroll
        for (int k = 0; k < NQ; ++k) s_c[k][tid] = acc[k];
    } else if (ci >= 0 && ci < S.nx && cj >= 0 && cj < S.ny) {
        const CellGeo g = geo_of(G, lx + 1, ly + 1);
        float V0 = 0.0f;
        if (REINIT) {
            const int cnt = count_cell(S, ci, cj, g);
            if (cnt) V0 = fdv(S.vol_el, (float)cnt);
        }
        visit_cell(S, ci, cj, g, [&](int q) {
            const float m = REINIT ? fm(V0, rho[q]) : S.mass[q];
            float cc[NQ];
            mass_contrib(S.x[q], S.y[q], S.vx[q], S.vy[q], m, g.cx, g.rx, g.cy, g.ry, cc);
            #pragma unroll
            for (int k = 0; k < NQ; ++k) s_c[k][tid] = fa(s_c[k][tid], cc[k]);
        });
    }
    __syncthreads();
    if (node_ok) {
        const float mass = node_sum(s_c + 0, tid);
        const float pxn = flush(node_sum(s_c + 4, tid));
        const float pyn = flush(node_sum(s_c + 8, tid));
        float vx, vy;
        if (mass == 0.0f) {
            vx = S.nvbx[node];
            vy = S.nvby[node];
        } else {
            vx = fdv(pxn, mass);
            vy = fdv(pyn, mass);
        }
        vx = flush(vx);
        vy = flush(vy);
        apply_constraint(S, ncons, vx, vy, nullptr, nullptr);
        S.nm[node] = mass;
        S.nvax[node] = vx;
        S.nvay[node] = vy;
    }
}

template <bool REINIT, int MINB = TILE_CTAS_LIGHT>
__global__ void __launch_bounds__(TILE_THREADS, MINB)
k_nodal_kinematics(const __grid_constant__ SimDev S, const int4* __restrict__ tiles,
                   Control* __restrict__ ctl, int k) {
    const int4 T = tiles[blockIdx.x];
    if (T.x < 0) return;   // past the active tiles
    nodal_kinematics_tile<REINIT>(S, T, ctl, k);
}

template <bool REINIT, int MINB = TILE_CTAS_LIGHT>
__global__ void __launch_bounds__(TILE_THREADS, MINB)
k_nodal_kinematics_batch(const TileDesc* __restrict__ td, int k) {
    __shared__ TileDesc sT;
    load_tile(td + blockIdx.x, sT);
    if (sT.T.x < 0) return;   // past the listed tiles
    nodal_kinematics_tile<REINIT, true>(sT.S, sT.T, sT.ctl, k, &sT);
}

// Nodal update shared by both schemes: concentrated forces (element.py:270-284),
// a = nan_to_num(f/m), v += a dt, constraints, flush (element.py:305-329).
// (fx, fy) is the summed internal plus external force of the particles.
// f / 0 after nan_to_num, exactly as nan_to_num(fdv(f, +0)) gives it
// (+-FLT_MAX for a force of that sign, 0 for a zero or NaN force), without
// the division's special-case path.
__device__ __forceinline__ float massless_accel(float f) {
    return f > 0.0f ? FLT_MAX : (f < 0.0f ? -FLT_MAX : 0.0f);
}

// MASSLESS: the node's mass is +0 (a node of an empty tile).
template <bool VD = false, bool MASSLESS = false>
__device__ __forceinline__ void nodal_update(const SimDev& S, int n, float t, float fx, float fy,
                                             float v0x, float v0y, float mass, uint16_t ncons) {
    if (rd<VD>(S.cnf_ptr)) {
        const int b = S.cnf_ptr[n], e = S.cnf_ptr[n + 1];
        #pragma unroll 1
        for (int k = b; k < e; ++k) {
            const float val = fm(fn_value(S, S.cnf_fn[k], t), S.cnf_val[k]);
            if (S.cnf_dir[k] == 0) fx = fa(fx, val);
            else fy = fa(fy, val);
        }
    }
    const float tx = fa(fx, 0.0f);   // + f_damp (zero, node.py:71)
    const float ty = fa(fy, 0.0f);
    float ax = MASSLESS ? massless_accel(tx) : nan_to_num(fdv(tx, mass));
    float ay = MASSLESS ? massless_accel(ty) : nan_to_num(fdv(ty, mass));
    const float dt = rd<VD>(S.dt);
    float vx = fa(v0x, fm(ax, dt));
    float vy = fa(v0y, fm(ay, dt));
    apply_constraint<VD>(S, ncons, vx, vy, &ax, &ay);
    rd<VD>(S.nvbx)[n] = flush(vx);
    rd<VD>(S.nvby)[n] = flush(vy);
    rd<VD>(S.nax)[n] = flush(ax);
    rd<VD>(S.nay)[n] = flush(ay);
}

// ---------------------------------------------------------------------------
// Phase 2 (USF): strain, volume and stress update (scheme.py:31-35 ->
// particle.py:249-327, material.py), external and internal forces
// (scheme.py:37-56 -> element.py:204-303, 842-901) and the nodal update
// (element.py:305-329).
// Phase 2 (USL): forces and nodal update only; the stress update runs after
// G2P (scheme.py:127-133).
// ---------------------------------------------------------------------------
constexpr int NV_W = TILE_CX + 1;   // node tile of the R cells: [c0x, c0x+33) x [c0y, c0y+17)
constexpr int NV_H = TILE_CY + 1;
constexpr int K2_ROW_P = 64;    // particles of a row per pass (measured against 32, 128 and 136)

// Fast paths of the forces kernel (StepConfig.forces_lpc):
//   FM_ROW     a warp's lanes take consecutive particles of its cell row
//              (coalesced global loads and stores); the contributions go
//              through shared-memory slots and lane l adds the slots of its
//              cell's particles in storage order.
//   FM_LPC     lane per cell: every lane works through its own cell's
//              particles in storage order, reading and writing them in
//              global memory, with the cell's nodal velocities and values in
//              registers, adding each contribution as it is formed.
//   FM_STAGED  FM_ROW on the cell row staged in shared memory by 16-byte
//              cp.async copies, one round trip per row instead of one per
//              particle a lane takes; a particle's contributions go to its
//              own staged slots once it has read them.
// All three add the same contributions in the same order: the same bits.
enum ForcesMode { FM_ROW = 0, FM_LPC = 1, FM_STAGED = 2 };

// Row-pass buffers of FM_ROW.
template <int NQ>
struct ForceRows {
    float slot[TILE_CY][NQ][K2_ROW_P];    // contributions of a row's particles
    unsigned char cell[TILE_CY][K2_ROW_P];   // their cell within the row
    float cellv[TILE_CY][3][32];          // V0, size0, dvol per cell
};

// Fields of the FM_STAGED row buffer: x, y and the stress state the forces
// use, then (USF) the rest of the state the step updates.  Slots 0..7 take a
// particle's eight contributions after it has read its fields.
template <bool USL, bool REINIT>
struct StagedFields {
    static constexpr int X = 0, Y = 1, SXX = 2, SYY = 3, SXY = 4, RHO = 5;
    static constexpr int SZZ = 6, EXX = 7, EYY = 8, EXY = 9, VSC = 10;   // USF only
    static constexpr int NBASE = USL ? 6 : 11;
    static constexpr int VOL = REINIT ? -1 : NBASE;   // solve semantics: persistent volume
    static constexpr int NF = NBASE + (REINIT ? 0 : 1);
    static constexpr int NBUF = NF > 8 ? NF : 8;
    // slots of a row per pass: a row of 4 particles in each of 32 cells,
    // starting anywhere in a 16-byte piece, fits one pass
    static constexpr int P = 132;
};

// Shared memory of forces_tile by mode.  FM_STAGED overlays the per-cell
// corner sums on the staged rows (they are formed after every row is done).
template <int MODE, int NQ, bool USL, bool REINIT>
struct ForceShared {
    float c[NQ][SC_STRIDE];
    ForceRows<NQ> rows;
};
template <int NQ, bool USL, bool REINIT>
struct ForceShared<FM_LPC, NQ, USL, REINIT> {
    float c[NQ][SC_STRIDE];
};
template <int NQ, bool USL, bool REINIT>
struct ForceShared<FM_STAGED, NQ, USL, REINIT> {
    using F = StagedFields<USL, REINIT>;
    union {
        float c[NQ][SC_STRIDE];
        __align__(16) float buf[TILE_CY][F::NBUF][F::P];
    };
    unsigned char cell[TILE_CY][F::P];   // a staged particle's cell within the row
    float cellv[TILE_CY][3][32];          // V0, size0, dvol per cell
    const float* src[F::NF];              // the staged fields' arrays (this step's parity)
};

// The arrays of the FM_STAGED fields, one per thread tid < NF.
template <bool USL, bool REINIT, bool VD>
__device__ __forceinline__ void staged_arrays(const SimDev& S, int parity, int tid, const float** src) {
    using F = StagedFields<USL, REINIT>;
    if (tid >= F::NF) return;
    const float* a = nullptr;
    switch (tid) {
        case F::X: a = rd<VD>(S.x); break;
        case F::Y: a = rd<VD>(S.y); break;
        case F::SXX: a = rd<VD>(S.sxx[parity]); break;
        case F::SYY: a = rd<VD>(S.syy[parity]); break;
        case F::SXY: a = rd<VD>(S.sxy[parity]); break;
        case F::RHO: a = rd<VD>(S.rho[parity]); break;
        default: break;
    }
    if constexpr (!USL) {
        switch (tid) {
            case F::SZZ: a = rd<VD>(S.szz[parity]); break;
            case F::EXX: a = rd<VD>(S.exx); break;
            case F::EYY: a = rd<VD>(S.eyy); break;
            case F::EXY: a = rd<VD>(S.exy); break;
            case F::VSC: a = rd<VD>(S.vsc[parity]); break;
            default: break;
        }
    }
    if constexpr (!REINIT) {
        if (tid == F::VOL) a = rd<VD>(S.vol[parity]);
    }
    src[tid] = a;
}

template <bool USL, bool REINIT, bool TRAC, bool VD, int MODE = FM_ROW>
__device__ __forceinline__ void forces_tile(const SimDev& S, const int4 T,
                                            Control* __restrict__ ctl, int k,
                                            const TileDesc* rec = nullptr) {
    constexpr int NQ = 8;
    __shared__ __align__(16) ForceShared<MODE, NQ, USL, REINIT> sh;
    auto& s_c = sh.c;                                   // [f x, f y] x corner, per cell
    __shared__ int s_cs[TILE_CY][33];
    __shared__ float2 s_v[NV_W * NV_H];   // nodal velocity after phase 1 of the tile's nodes
    __shared__ TileGeo G;
    const int step = load_step(ctl) + k;
    const int parity = step & 1;
    const float t = step_time(step, S.dt);
    const int tid = threadIdx.x, lx = tid & (TILE_CX - 1), ly = tid / TILE_CX;
    const int c0x = T.y * TILE_NX - 1, c0y = T.z * TILE_NY - 1;
    const int ci = c0x + lx, cj = c0y + ly;
    const bool node_ok = lx < TILE_NX && ly < TILE_NY && c0x + 1 + lx <= S.nx && c0y + 1 + ly <= S.ny;
    const int node = (c0y + 1 + ly) * (S.nx + 1) + c0x + 1 + lx;
    // node-phase inputs, fetched early
    const float nmass = node_ok ? S.nm[node] : 0.0f;
    const uint16_t ncons = node_ok ? S.ncons[node] : 0;
    // the node tile (two entries per thread at most) and the tile set-up in
    // one round trip
    static_assert(NV_W * NV_H <= 2 * TILE_THREADS, "two node-tile entries per thread");
    float2 nv[2];
    #pragma unroll
    for (int e = 0; e < 2; ++e) {
        const int idx = tid + e * TILE_THREADS;
        const int I = c0x + idx % NV_W, J = c0y + idx / NV_W;
        nv[e] = make_float2(0.0f, 0.0f);
        if (idx < NV_W * NV_H && I >= 0 && I <= S.nx && J >= 0 && J <= S.ny) {
            const int n = J * (S.nx + 1) + I;
            nv[e] = make_float2(S.nvax[n], S.nvay[n]);
        }
    }
    const TileLoads L = VD ? record_loads(S, *rec, c0x, c0y, ly, lx) : tile_loads(S, c0x, c0y, cj, lx);
    if (!__syncthreads_or(L.occ)) {
        // no particle in the tile: the nodal update with zero particle forces
        if (node_ok) nodal_update<VD>(S, node, t, 0.0f, 0.0f, S.nvax[node], S.nvay[node], nmass, ncons);
        return;
    }
    build_geo(S, c0x, c0y, G);
    if constexpr (MODE != FM_STAGED) {
        #pragma unroll
        for (int q = 0; q < NQ; ++q) s_c[q][tid] = 0.0f;
    }
    s_cs[ly][lx] = L.cs;
    if (lx == 0) s_cs[ly][32] = L.cs32;
    #pragma unroll
    for (int e = 0; e < 2; ++e)
        if (tid + e * TILE_THREADS < NV_W * NV_H) s_v[tid + e * TILE_THREADS] = nv[e];
    if constexpr (MODE == FM_STAGED) staged_arrays<USL, REINIT, VD>(S, parity, tid, sh.src);
    if constexpr (!USL) stage_materials<VD>(S);
    const bool slow = __syncthreads_or(L.drift) != 0;

    auto cell_velocities = [&](int li, int lj, float* vx, float* vy) {
        const int a = lj * NV_W + li;
        const int id[4] = {a, a + 1, a + NV_W + 1, a + NV_W};
        #pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float2 v = s_v[id[k]];
            vx[k] = v.x;
            vy[k] = v.y;
        }
    };

    if (!slow) {
      if constexpr (MODE == FM_STAGED) {
        using F = StagedFields<USL, REINIT>;
        float (*buf)[F::P] = sh.buf[ly];
        auto& s_cell = sh.cell;
        auto& s_cellv = sh.cellv;
        const int* cs = s_cs[ly];
        const int rb = cs[0], re = cs[32], cb = cs[lx], ce = cs[lx + 1];
        {
            float nvx[4], nvy[4], V0, size0, dvol;
            if (!USL) cell_velocities(lx, ly, nvx, nvy);
            force_cell_values<USL, REINIT, VD, TRAC>(S, ce - cb, geo_of(G, lx + 1, ly + 1), nvx, nvy, V0,
                                                     size0, dvol);
            s_cellv[ly][0][lx] = V0;
            s_cellv[ly][1][lx] = size0;
            s_cellv[ly][2][lx] = dvol;
        }
        const float cy = G.row[ly + 1].z, ry = G.row[ly + 1].w;   // row geometry (warp-uniform)
        const int next = parity ^ 1;
        float acc[NQ];
        #pragma unroll
        for (int q = 0; q < NQ; ++q) acc[q] = 0.0f;
        #pragma unroll 1
        for (int p0 = rb & ~3; p0 < re; p0 += F::P) {
            const int p1 = min(p0 + F::P, re);
            #pragma unroll
            for (int f = 0; f < F::NF; ++f) {
                #pragma unroll
                for (int o = 4 * lx; o < F::P; o += 128)
                    if (p0 + o < p1) cp_async16(&buf[f][o], sh.src[f] + p0 + o);
            }
            cp_async_commit();
            for (int q = max(cb, p0); q < min(ce, p1); ++q) s_cell[ly][q - p0] = (unsigned char)lx;
            cp_async_wait<0>();
            __syncwarp();
            #pragma unroll 1
            for (int q = max(rb, p0) + lx; q < p1; q += 32) {
                const int j = q - p0;
                const int l = s_cell[ly][j];
                float nvx[4], nvy[4];
                if (!USL) cell_velocities(l, ly, nvx, nvy);
                PState p;
                p.sxx = buf[F::SXX][j];
                p.syy = buf[F::SYY][j];
                p.sxy = buf[F::SXY][j];
                p.rho = buf[F::RHO][j];
                p.szz = 0.0f;
                if constexpr (!USL) {
                    p.szz = buf[F::SZZ][j];
                    p.exx = buf[F::EXX][j];
                    p.eyy = buf[F::EYY][j];
                    p.exy = buf[F::EXY][j];
                    p.vsc = buf[F::VSC][j];
                }
                const float4 cg = G.col[l + 1];
                float cc[NQ];
                const float V = force_core<USL, REINIT, TRAC, VD>(
                    S, q, buf[F::X][j], buf[F::Y][j], p, REINIT ? s_cellv[ly][0][l] : buf[REINIT ? 0 : F::VOL][j],
                    cg.z, cg.w, cy, ry, s_cellv[ly][1][l], nvx, nvy, s_cellv[ly][2][l], t, cc);
                if (!USL && l >= 1 && ly >= 1) store_state<REINIT, VD>(S, q, p, V, next);
                #pragma unroll
                for (int kk = 0; kk < NQ; ++kk) buf[kk][j] = cc[kk];
            }
            __syncwarp();
            #pragma unroll 1
            for (int q = max(cb, p0); q < min(ce, p1); ++q) {
                #pragma unroll
                for (int kk = 0; kk < NQ; ++kk) acc[kk] = fa(acc[kk], buf[kk][q - p0]);
            }
            __syncwarp();
        }
        __syncthreads();   // every row is done with the staged rows that s_c overlays
        #pragma unroll
        for (int q = 0; q < NQ; ++q) s_c[q][tid] = acc[q];
      } else if constexpr (MODE == FM_LPC) {
        if (ci >= 0 && ci < S.nx && cj >= 0 && cj < S.ny) {
            const int cb = s_cs[ly][lx], ce = s_cs[ly][lx + 1];
            const CellGeo g = geo_of(G, lx + 1, ly + 1);
            float nvx[4], nvy[4], V0, size0, dvol;
            if (!USL) cell_velocities(lx, ly, nvx, nvy);
            force_cell_values<USL, REINIT, VD, TRAC>(S, ce - cb, g, nvx, nvy, V0, size0, dvol);
            const bool own = lx >= 1 && ly >= 1;
            float acc[NQ];
            #pragma unroll
            for (int q = 0; q < NQ; ++q) acc[q] = 0.0f;
            #pragma unroll 1
            for (int q = cb; q < ce; ++q) {
                float cc[NQ];
                force_contrib<USL, REINIT, TRAC, VD>(S, q, force_in_global<VD>(S, q, parity, REINIT), g.cx,
                                                     g.rx, g.cy, g.ry, V0, size0, nvx, nvy, dvol, parity,
                                                     t, own, cc);
                #pragma unroll
                for (int kk = 0; kk < NQ; ++kk) acc[kk] = fa(acc[kk], cc[kk]);
            }
            #pragma unroll
            for (int q = 0; q < NQ; ++q) s_c[q][tid] = acc[q];
        }
      } else {
        // particle per lane for the per-particle work (coalesced global loads
        // and stores), contributions to row slots, then lane per cell adds
        // the slots of its cell's particles in storage order
        auto& s_slot = sh.rows.slot;
        auto& s_cell = sh.rows.cell;
        auto& s_cellv = sh.rows.cellv;
        const int* cs = s_cs[ly];
        const int rb = cs[0], re = cs[32];
        const int cb = cs[lx], ce = cs[lx + 1];
        {
            float nvx[4], nvy[4], V0, size0, dvol;
            if (!USL) cell_velocities(lx, ly, nvx, nvy);
            force_cell_values<USL, REINIT, VD, TRAC>(S, ce - cb, geo_of(G, lx + 1, ly + 1), nvx, nvy, V0,
                                           size0, dvol);
            s_cellv[ly][0][lx] = V0;
            s_cellv[ly][1][lx] = size0;
            s_cellv[ly][2][lx] = dvol;
        }
        const float cy = G.row[ly + 1].z, ry = G.row[ly + 1].w;   // row geometry (warp-uniform)
        float acc[NQ];
        #pragma unroll
        for (int k = 0; k < NQ; ++k) acc[k] = 0.0f;
        #pragma unroll 1
        for (int p0 = rb; p0 < re; p0 += K2_ROW_P) {
            const int p1 = min(p0 + K2_ROW_P, re);
            for (int q = max(cb, p0); q < min(ce, p1); ++q) s_cell[ly][q - p0] = (unsigned char)lx;
            __syncwarp();
            #pragma unroll 1
            for (int q = p0 + lx; q < p1; q += 32) {
                const int l = s_cell[ly][q - p0];
                float nvx[4], nvy[4];
                if (!USL) cell_velocities(l, ly, nvx, nvy);
                float cc[NQ];
                force_contrib<USL, REINIT, TRAC, VD>(S, q, force_in_global<VD>(S, q, parity, REINIT),
                                                 G.col[l + 1].z, G.col[l + 1].w, cy, ry,
                                                 s_cellv[ly][0][l], s_cellv[ly][1][l], nvx, nvy,
                                                 s_cellv[ly][2][l], parity, t, l >= 1 && ly >= 1,
                                                 cc);
                #pragma unroll
                for (int k = 0; k < NQ; ++k) s_slot[ly][k][q - p0] = cc[k];
            }
            __syncwarp();
            #pragma unroll 1
            for (int q = max(cb, p0); q < min(ce, p1); ++q) {
                #pragma unroll
                for (int k = 0; k < NQ; ++k) acc[k] = fa(acc[k], s_slot[ly][k][q - p0]);
            }
            __syncwarp();
        }
        #pragma unroll
        for (int k = 0; k < NQ; ++k) s_c[k][tid] = acc[k];
      }
    } else {
        if constexpr (MODE == FM_STAGED) {
            #pragma unroll
            for (int q = 0; q < NQ; ++q) s_c[q][tid] = 0.0f;
        }
        if (ci >= 0 && ci < S.nx && cj >= 0 && cj < S.ny) {
            const CellGeo g = geo_of(G, lx + 1, ly + 1);
            const int cnt = REINIT ? count_cell(S, ci, cj, g) : 0;
            float nvx[4], nvy[4], V0, size0, dvol;
            if (!USL) cell_velocities(lx, ly, nvx, nvy);
            force_cell_values<USL, REINIT, VD, TRAC>(S, cnt, g, nvx, nvy, V0, size0, dvol);
            const bool own = lx >= 1 && ly >= 1;
            visit_cell(S, ci, cj, g, [&](int q) {
                float cc[NQ];
                force_contrib<USL, REINIT, TRAC, VD>(S, q, force_in_global<VD>(S, q, parity, REINIT), g.cx,
                                                 g.rx, g.cy, g.ry, V0, size0, nvx, nvy, dvol, parity,
                                                 t, own, cc);
                #pragma unroll
                for (int k = 0; k < NQ; ++k) s_c[k][tid] = fa(s_c[k][tid], cc[k]);
            });
        }
    }
    __syncthreads();
    if (node_ok) {
        const int a = (ly + 1) * NV_W + lx + 1;   // node (I, J) in the node tile
        nodal_update<VD>(S, node, t, node_sum(s_c + 0, tid), node_sum(s_c + 4, tid), s_v[a].x, s_v[a].y,
                     nmass, ncons);
    }
}

template <bool USL, bool REINIT, bool TRAC, int MODE = FM_ROW>
__global__ void __launch_bounds__(TILE_THREADS, TILE_MIN_CTAS)
k_forces(const __grid_constant__ SimDev S, const int4* __restrict__ tiles,
         Control* __restrict__ ctl, int k) {
    const int4 T = tiles[blockIdx.x];
    if (T.x < 0) return;
    forces_tile<USL, REINIT, TRAC, false, MODE>(S, T, ctl, k);
}

template <bool USL, bool REINIT, bool TRAC, int MODE = FM_ROW>
__global__ void __launch_bounds__(TILE_THREADS, TILE_MIN_CTAS)
k_forces_batch(const TileDesc* __restrict__ td, int k) {
    __shared__ TileDesc sT;
    load_tile(td + blockIdx.x, sT);
    if (sT.T.x < 0) return;   // past the listed tiles
    forces_tile<USL, REINIT, TRAC, true, MODE>(sT.S, sT.T, sT.ctl, k, &sT);
}

// ---------------------------------------------------------------------------
// Phase 3: G2P (diffmpm/particle.py:208-247): v_hat = sum N v_i,
// a_hat = sum N a_i, v_p = v_hat or v_p + a_hat dt, x_p += v_hat dt.  USL adds
// the strain/volume/stress update at the step's natural coordinates with the
// updated nodal velocities (scheme.py:127-133).  Warp w streams the particles
// of the owned sort-cells of row w + 1 (one particle per lane, staged with
// cp.async) against a shared-memory tile of the nodal velocity and
// acceleration, and records per sort-cell whether a particle now lies in
// another cell (the drift flags).
// ---------------------------------------------------------------------------
constexpr int G_W = TILE_CX + 2;   // node tile [c0x, c0x+34) x [c0y, c0y+18)
constexpr int G_H = TILE_CY + 2;
constexpr int G2P_MAP = 160;        // particles of a row whose sort-cell is looked up in a map

// New cell along one axis for a coordinate that was in table column k (cell
// c = base + k): same, or a neighbour by one, decided against the tabulated
// bounds; otherwise a full locate.
__device__ __forceinline__ int moved_axis(float x, const float4* tab, int k, int nk, int c, float h,
                                          int n) {
    const float lo = tab[k].x, hi = tab[k].y;
    if (x >= lo && x < hi) return c;
    if (x >= hi && k + 1 < nk && x < tab[k + 1].y) return c + 1;
    if (x < lo && k >= 1 && x >= tab[k - 1].x) return c - 1;
    return locate_axis(x, h, n);
}

enum G2PField { GF_X, GF_Y, GF_VX, GF_VY, GF_SXX, GF_SYY, GF_SZZ, GF_SXY, GF_EXX, GF_EYY,
                GF_EXY, GF_RHO, GF_VSC, GF_VOL, GF_N };

template <bool USL>
struct G2PStage {
    static constexpr int NF = USL ? GF_N : 4;
    static constexpr int DEPTH = USL ? 2 : 4;
};

// Per-warp staging of a row's particles in chunks of 32 storage slots that
// start on 16-byte boundaries: chunk c holds slots rb4 + 32c + [0, 32) with
// rb4 = rb rounded down to a multiple of 4, copied as 16-byte cp.async pieces
// (8 per field; NF = 4 fields is one piece per lane).  Pieces wholly past the
// row end re are skipped; the last piece may read up to 3 slots past re,
// which the particle arrays' padding (a multiple of 4 slots) covers.  Slot q
// of chunk c lands in buf[c % DEPTH][f][q - rb4 - 32c].
template <int NF, int DEPTH>
struct RowStage16 {
    static constexpr int NP = (NF * 8 + 31) / 32;   // pieces per lane per chunk
    float* buf;                 // [DEPTH][NF][32]
    const float* lp[NP];        // this lane's source array for its piece j (null: none)
    int doff[NP];               // and its offset in a chunk's [NF][32] block
    int lo, rb4, re, nch;

    // src: the NF source arrays (null entries are not staged)
    __device__ __forceinline__ RowStage16(float* b, const float* const* src, int rb, int re_, int lane)
        : buf(b), lo((lane & 7) * 4), rb4(rb & ~3), re(re_), nch(re_ > rb ? (re_ - (rb & ~3) + 31) / 32 : 0) {
        #pragma unroll
        for (int j = 0; j < NP; ++j) {
            const int p = 32 * j + lane, f = p >> 3;
            // select the field without indexing src by a runtime value
            const float* ptr = nullptr;
            #pragma unroll
            for (int g = 4 * j; g < 4 * j + 4 && g < NF; ++g)
                if (f == g) ptr = src[g];
            lp[j] = p < NF * 8 ? ptr : nullptr;
            doff[j] = f * 32 + lo;
        }
    }
    __device__ __forceinline__ void issue(int c) {
        if (c < nch) {
            const int base = rb4 + 32 * c + lo;
            float* dst = buf + (c % DEPTH) * (NF * 32);
            #pragma unroll
            for (int j = 0; j < NP; ++j)
                if (lp[j] && base < re) cp_async16(dst + doff[j], lp[j] + base);
        }
        cp_async_commit();
    }
    __device__ __forceinline__ void prime() {
        #pragma unroll
        for (int c = 0; c < DEPTH - 1; ++c) issue(c);
    }
    // Issue chunk c + DEPTH - 1 and wait until chunk c has landed (visible to
    // the whole warp).
    __device__ __forceinline__ const float (*advance(int c))[32] {
        issue(c + DEPTH - 1);
        cp_async_wait<DEPTH - 1>();
        __syncwarp();
        return reinterpret_cast<const float (*)[32]>(buf + (c % DEPTH) * (NF * 32));
    }
};

// G2P of one particle (storage slot q, staged inputs b[.][lane]) in cell
// (ci, cj) with geometry g and corner nodal values nd[4] = (vx, vy, ax, ay):
// velocity and position update (particle.py:208-247) and, under USL, the
// strain/volume/stress update (scheme.py:127-133).  Writes the particle and
// returns the new position.
template <bool USL, bool REINIT>
__device__ __forceinline__ float2 g2p_particle(const SimDev& S, int q, const float (*b)[32], int lane,
                                               const CellGeo& g, const float4 nd[4], int next) {
    const float dt = S.dt;
    const float x = b[GF_X][lane], y = b[GF_Y][lane];
    const float xi = natural(x, g.cx, g.rx);
    const float eta = natural(y, g.cy, g.ry);
    float N[4], nvx[4], nvy[4], nax[4], nay[4];
    shape4(xi, eta, N);
    #pragma unroll
    for (int k = 0; k < 4; ++k) {
        nvx[k] = nd[k].x;
        nvy[k] = nd[k].y;
        nax[k] = nd[k].z;
        nay[k] = nd[k].w;
    }
    const float vhx = dot4(N, nvx), vhy = dot4(N, nvy);
    float vx, vy;
    if (S.velocity_update) {
        vx = vhx;
        vy = vhy;
    } else {
        vx = fa(b[GF_VX][lane], fm(dot4(N, nax), dt));
        vy = fa(b[GF_VY][lane], fm(dot4(N, nay), dt));
    }
    if (S.pvc) {   // particle velocity constraints (an extension; scheme.py:67 leaves a TODO)
        const uchar2 c = reinterpret_cast<const uchar2*>(S.pvc)[q];
        if (c.x) vx = S.pvc_vel[c.x - 1];
        if (c.y) vy = S.pvc_vel[c.y - 1];
    }
    const float xn = fa(x, fm(vhx, dt)), yn = fa(y, fm(vhy, dt));
    S.x[q] = xn;
    S.y[q] = yn;
    S.vx[q] = vx;
    S.vy[q] = vy;
    if constexpr (USL) {
        float Gcx[4], Gcy[4], c0, c1, c3;
        dshape4(0.0f, 0.0f, g.rx, g.ry, Gcx, Gcy);
        strain_rate4(Gcx, Gcy, nvx, nvy, c0, c1, c3);
        const float dvol = fm(dt, fa(c0, c1));
        float Gx[4], Gy[4], r0, r1, r3;
        dshape4(xi, eta, g.rx, g.ry, Gx, Gy);
        strain_rate4(Gx, Gy, nvx, nvy, r0, r1, r3);
        PState p;
        p.sxx = b[GF_SXX][lane];
        p.syy = b[GF_SYY][lane];
        p.szz = b[GF_SZZ][lane];
        p.sxy = b[GF_SXY][lane];
        p.exx = b[GF_EXX][lane];
        p.eyy = b[GF_EYY][lane];
        p.exy = b[GF_EXY][lane];
        p.rho = b[GF_RHO][lane];
        p.vsc = b[GF_VSC][lane];
        const MatDev& M = material_of<false>(S, q);
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
        if (!REINIT) S.vol[next][q] = fm(b[GF_VOL][lane], f);
    }
    return make_float2(xn, yn);
}

template <bool USL, bool REINIT, bool REC = false>
__device__ __forceinline__ void particle_kinematics_tile(const SimDev& S, const int4 T,
                                                         Control* __restrict__ ctl, int k,
                                                         const TileDesc* rec = nullptr) {
    constexpr int NF = G2PStage<USL>::NF, DEPTH = G2PStage<USL>::DEPTH;
    __shared__ float4 s_nd[G_W * G_H];    // nodal (vx, vy, ax, ay) of the tile's nodes
    __shared__ __align__(16) float s_stage[TILE_CY][DEPTH][NF][32];
    __shared__ int s_cs[TILE_CY][33];
    __shared__ unsigned char s_map[TILE_CY][G2P_MAP];   // sort-cell of the row's first particles
    __shared__ int s_flag[TILE_CY][32];   // drift flag after this step
    __shared__ int s_status;
    __shared__ TileGeo G;
    const int step = load_step(ctl) + k;
    const int parity = step & 1, next = parity ^ 1;
    const int tid = threadIdx.x, lane = tid & 31, w = tid / 32;
    const int c0x = T.y * TILE_NX - 1, c0y = T.z * TILE_NY - 1;
    // row w + 1 of the tile: owned sort-cells c0x+1 .. c0x+31 -> starts cs[0..31]
    const int sj = c0y + 1 + w;
    const bool row_ok = w < TILE_NY && sj < S.ny;
    int rb = 0, re = 0;
    unsigned sfmask = 0;   // bit l: sort-cell c0x + 1 + l had a drifted particle at the step start
    if (row_ok) {
        // (a batched tile's row starts come with its record: row w + 1,
        // column lane + 1 of the record's table)
        const int col = min(c0x + 1 + lane, S.nx);
        s_cs[w][lane] = REC ? rec->cs[w + 1][lane + 1] : S.cstart[sj * S.nx + col];
        sfmask = __ballot_sync(0xffffffffu, col < S.nx && S.cflag[sj * S.nx + col] != 0);
    }
    s_flag[w][lane] = 0;
    __syncwarp();
    if (row_ok) {
        rb = s_cs[w][0];
        re = s_cs[w][31];
    }
    const float* src[NF] = {S.x, S.y, S.vx, S.vy};
    if constexpr (USL) {
        src[GF_SXX] = S.sxx[parity];
        src[GF_SYY] = S.syy[parity];
        src[GF_SZZ] = S.szz[parity];
        src[GF_SXY] = S.sxy[parity];
        src[GF_EXX] = S.exx;
        src[GF_EYY] = S.eyy;
        src[GF_EXY] = S.exy;
        src[GF_RHO] = S.rho[parity];
        src[GF_VSC] = S.vsc[parity];
        src[GF_VOL] = REINIT ? nullptr : S.vol[parity];
    }
    RowStage16<NF, DEPTH> st(&s_stage[w][0][0][0], src, rb, re, lane);
    const int rb4 = st.rb4;
    st.prime();
    if constexpr (USL) stage_materials<false>(S);
    if (!__syncthreads_or(re > rb)) {
        // no particle stored in the tile's sort-cells: their drift flags clear
        if (row_ok && lane < TILE_NX && c0x + 1 + lane < S.nx) S.cflag[sj * S.nx + c0x + 1 + lane] = 0;
        return;
    }
    if (tid == 0) s_status = 0;
    {
        // the node tile, both entries of a thread in flight together (and in
        // flight with the rows' first chunks)
        static_assert(G_W * G_H <= 2 * TILE_THREADS, "two node-tile entries per thread");
        float4 nd[2];
        #pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int idx = tid + e * TILE_THREADS;
            const int I = c0x + idx % G_W, J = c0y + idx / G_W;
            nd[e] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (idx < G_W * G_H && I >= 0 && I <= S.nx && J >= 0 && J <= S.ny) {
                const int n = J * (S.nx + 1) + I;
                nd[e] = make_float4(S.nvbx[n], S.nvby[n], S.nax[n], S.nay[n]);
            }
        }
        build_geo(S, c0x, c0y, G);
        #pragma unroll
        for (int e = 0; e < 2; ++e)
            if (tid + e * TILE_THREADS < G_W * G_H) s_nd[tid + e * TILE_THREADS] = nd[e];
    }
    if (row_ok && lane < TILE_NX) {
        // storage index rb + j of the row holds a particle of sort-cell s_map[j]
        const int lo = s_cs[w][lane] - rb, hi = min(s_cs[w][lane + 1] - rb, G2P_MAP);
        for (int j = lo; j < hi; ++j) s_map[w][j] = (unsigned char)lane;
    }
    __syncthreads();
    int status = 0;
    const int* cs = s_cs[w];
    // this row's geometry (a particle still in its sort-cell is in row sj)
    const float4 rg = G.row[w + 2];
    const float4* nrow = s_nd + (w + 1) * G_W + 1;   // node (c0x + 1, sj) of the node tile
    #pragma unroll 1
    for (int c = 0; c < st.nch; ++c) {
        const float (*b)[32] = st.advance(c);
        const int q = rb4 + 32 * c + lane;
        if (q < rb || q >= re) continue;
        const int l = q - rb < G2P_MAP ? s_map[w][q - rb] : cell_of(cs, 30, q);   // sort-cell c0x + 1 + l
        if (!((sfmask >> l) & 1u)) {
            // fast path: the particle is in its sort-cell (c0x + 1 + l, sj)
            const float4 cg = G.col[l + 2];
            CellGeo g;
            g.x0 = cg.x;
            g.x1 = cg.y;
            g.cx = cg.z;
            g.rx = cg.w;
            g.y0 = rg.x;
            g.y1 = rg.y;
            g.cy = rg.z;
            g.ry = rg.w;
            const float4* a = nrow + l;
            const float4 nd[4] = {a[0], a[1], a[G_W + 1], a[G_W]};
            const float2 pn = g2p_particle<USL, REINIT>(S, q, b, lane, g, nd, next);
            if (!(pn.x >= g.x0 && pn.x < g.x1 && pn.y >= g.y0 && pn.y < g.y1)) {
                const int si = c0x + 1 + l;
                const int ni = moved_axis(pn.x, G.col, l + 2, GEO_C, si, S.hx, S.nx);
                const int nj = moved_axis(pn.y, G.row, w + 2, GEO_R, sj, S.hy, S.ny);
                s_flag[w][l] = 1;
                if (ni < 0 || ni >= S.nx || nj < 0 || nj >= S.ny) status |= ST_OUT_OF_MESH;
                else if (max(abs(ni - si), abs(nj - sj)) > 1) status |= ST_DRIFT_VIOLATION;
            }
            continue;
        }
        // the sort-cell holds drifted particles: locate this one
        const int si = c0x + 1 + l;
        const float x = b[GF_X][lane], y = b[GF_Y][lane];
        const int ci = locate_axis(x, S.hx, S.nx);
        const int cj = locate_axis(y, S.hy, S.ny);
        if (ci < 0 || ci >= S.nx || cj < 0 || cj >= S.ny) {
            status |= ST_OUT_OF_MESH;
            s_flag[w][l] = 1;
            continue;
        }
        const int kc = ci - c0x + 1, kr = cj - c0y + 1;   // geometry table indices
        const bool in_tile = kc >= 0 && kc < GEO_C && kr >= 0 && kr < GEO_R;
        const CellGeo g = in_tile ? geo_of(G, kc, kr) : cell_geo(ci, cj, S.hx, S.hy);
        float4 nd[4];
        const int li = ci - c0x, lj = cj - c0y;
        if (li >= 0 && li + 1 < G_W && lj >= 0 && lj + 1 < G_H) {
            const int a = lj * G_W + li;
            nd[0] = s_nd[a];
            nd[1] = s_nd[a + 1];
            nd[2] = s_nd[a + G_W + 1];
            nd[3] = s_nd[a + G_W];
        } else {
            int ids[4];
            cell_nodes(S, ci, cj, ids);
            #pragma unroll
            for (int kk = 0; kk < 4; ++kk)
                nd[kk] = make_float4(S.nvbx[ids[kk]], S.nvby[ids[kk]], S.nax[ids[kk]], S.nay[ids[kk]]);
        }
        const float2 pn = g2p_particle<USL, REINIT>(S, q, b, lane, g, nd, next);
        int ni, nj;
        if (in_tile) {
            ni = moved_axis(pn.x, G.col, kc, GEO_C, ci, S.hx, S.nx);
            nj = moved_axis(pn.y, G.row, kr, GEO_R, cj, S.hy, S.ny);
        } else {
            ni = locate_axis(pn.x, S.hx, S.nx);
            nj = locate_axis(pn.y, S.hy, S.ny);
        }
        if (ni < 0 || ni >= S.nx || nj < 0 || nj >= S.ny) {
            status |= ST_OUT_OF_MESH;
            s_flag[w][l] = 1;
        } else {
            const int d = max(abs(ni - si), abs(nj - sj));
            if (d >= 1) s_flag[w][l] = 1;
            if (d > 1) status |= ST_DRIFT_VIOLATION;
        }
    }
    cp_async_wait<0>();
    __syncwarp();
    if (row_ok && lane < TILE_NX) {
        const int si = c0x + 1 + lane;
        if (si < S.nx) {
            const int f = s_flag[w][lane];
            S.cflag[sj * S.nx + si] = (uint8_t)f;
            if (f) status |= ST_DRIFTED;
        }
    }
    // block-wide OR of the status bits, then one atomic per CTA
    status = __reduce_or_sync(0xffffffffu, status);
    if (lane == 0 && status) atomicOr(&s_status, status);
    __syncthreads();
    if (tid == 0 && s_status) atomicOr(&ctl->status, s_status);
}

template <bool USL, bool REINIT, int MINB = (USL ? TILE_MIN_CTAS : TILE_CTAS_LIGHT)>
__global__ void __launch_bounds__(TILE_THREADS, MINB)
k_particle_kinematics(const __grid_constant__ SimDev S, const int4* __restrict__ tiles,
                      Control* __restrict__ ctl, int k) {
    const int4 T = tiles[blockIdx.x];
    if (T.x < 0) return;
    particle_kinematics_tile<USL, REINIT>(S, T, ctl, k);
}

template <bool USL, bool REINIT, int MINB = (USL ? TILE_MIN_CTAS : TILE_CTAS_LIGHT)>
__global__ void __launch_bounds__(TILE_THREADS, MINB)
k_particle_kinematics_batch(const TileDesc* __restrict__ td, int k) {
    __shared__ TileDesc sT;
    load_tile(td + blockIdx.x, sT);
    if (sT.T.x < 0) return;   // past the listed tiles
    // no particle stored in the tile's sort-cells or around them: nothing
    // moves, and the sort-cells' drift flags are already clear (a flag is set
    // only for a sort-cell that stores a particle, and a re-sort clears all)
    if (!sT.occ) return;
    particle_kinematics_tile<USL, REINIT, true>(sT.S, sT.T, sT.ctl, k, &sT);
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
// The step kernels use 50-110 KB of shared memory per CTA and are sized for two
// or three CTAs per SM: ask for the largest shared-memory carveout once per kernel.
template <class K>
static void prefer_shared(K kernel) {
    static bool done = false;
    if (!done) {
        cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
        done = true;
    }
}

// The nodal kinematics and USF G2P kernels come in two builds: 40 registers
// and three CTAs per SM, or up to 64 registers and two (StepConfig.nk_ctas,
// g2p_ctas; chosen by the autotuner).
template <bool REINIT>
static void nodal_kinematics(const SimDev& S, const int4* tiles, int ntiles, Control* ctl,
                             int k, int ctas, cudaStream_t s) {
    if (ctas == 2) {
        prefer_shared(k_nodal_kinematics<REINIT, 2>);
        k_nodal_kinematics<REINIT, 2><<<ntiles, TILE_THREADS, 0, s>>>(S, tiles, ctl, k);
        return;
    }
    prefer_shared(k_nodal_kinematics<REINIT>);
    k_nodal_kinematics<REINIT><<<ntiles, TILE_THREADS, 0, s>>>(S, tiles, ctl, k);
}

cudaError_t launch_nodal_kinematics(const StepConfig& c, const SimDev& S, const int4* tiles,
                                    int ntiles, Control* ctl, int k, cudaStream_t s) {
    if (c.reinit) nodal_kinematics<true>(S, tiles, ntiles, ctl, k, c.nk_ctas, s);
    else nodal_kinematics<false>(S, tiles, ntiles, ctl, k, c.nk_ctas, s);
    return cudaGetLastError();
}

template <bool USL, bool REINIT, bool TRAC, int MODE>
static void forces_mode(const SimDev& S, const int4* tiles, int ntiles, Control* ctl, int k,
                        cudaStream_t s) {
    prefer_shared(k_forces<USL, REINIT, TRAC, MODE>);
    k_forces<USL, REINIT, TRAC, MODE><<<ntiles, TILE_THREADS, 0, s>>>(S, tiles, ctl, k);
}

template <bool USL, bool REINIT, bool TRAC>
static void forces_one(int mode, const SimDev& S, const int4* tiles, int ntiles, Control* ctl, int k,
                       cudaStream_t s) {
    if (mode == FM_STAGED) forces_mode<USL, REINIT, TRAC, FM_STAGED>(S, tiles, ntiles, ctl, k, s);
    else if (mode == FM_LPC) forces_mode<USL, REINIT, TRAC, FM_LPC>(S, tiles, ntiles, ctl, k, s);
    else forces_mode<USL, REINIT, TRAC, FM_ROW>(S, tiles, ntiles, ctl, k, s);
}

template <bool USL, bool REINIT>
static void forces_trac(bool trac, int lpc, const SimDev& S, const int4* tiles, int ntiles,
                        Control* ctl, int k, cudaStream_t s) {
    if (trac) forces_one<USL, REINIT, true>(lpc, S, tiles, ntiles, ctl, k, s);
    else forces_one<USL, REINIT, false>(lpc, S, tiles, ntiles, ctl, k, s);
}

cudaError_t launch_forces(const StepConfig& c, const SimDev& S, const int4* tiles, int ntiles,
                          Control* ctl, int k, cudaStream_t s) {
    const int lpc = c.forces_lpc;
    if (c.usl) {
        if (c.reinit) forces_trac<true, true>(c.traction, lpc, S, tiles, ntiles, ctl, k, s);
        else forces_trac<true, false>(c.traction, lpc, S, tiles, ntiles, ctl, k, s);
    } else {
        if (c.reinit) forces_trac<false, true>(c.traction, lpc, S, tiles, ntiles, ctl, k, s);
        else forces_trac<false, false>(c.traction, lpc, S, tiles, ntiles, ctl, k, s);
    }
    return cudaGetLastError();
}

template <bool USL, bool REINIT>
static void particle_kinematics(const SimDev& S, const int4* tiles, int ntiles, Control* ctl,
                                int k, int ctas, cudaStream_t s) {
    if (!USL && ctas == 2) {
        prefer_shared(k_particle_kinematics<USL, REINIT, 2>);
        k_particle_kinematics<USL, REINIT, 2><<<ntiles, TILE_THREADS, 0, s>>>(S, tiles, ctl, k);
        return;
    }
    prefer_shared(k_particle_kinematics<USL, REINIT>);
    k_particle_kinematics<USL, REINIT><<<ntiles, TILE_THREADS, 0, s>>>(S, tiles, ctl, k);
}

cudaError_t launch_particle_kinematics(const StepConfig& c, const SimDev& S, const int4* tiles,
                                       int ntiles, Control* ctl, int k, cudaStream_t s) {
    if (c.usl) {
        if (c.reinit) particle_kinematics<true, true>(S, tiles, ntiles, ctl, k, c.g2p_ctas, s);
        else particle_kinematics<true, false>(S, tiles, ntiles, ctl, k, c.g2p_ctas, s);
    } else {
        if (c.reinit) particle_kinematics<false, true>(S, tiles, ntiles, ctl, k, c.g2p_ctas, s);
        else particle_kinematics<false, false>(S, tiles, ntiles, ctl, k, c.g2p_ctas, s);
    }
    return cudaGetLastError();
}

// Batched launches: one grid over the tiles of every simulation of a batch.
template <bool REINIT>
static void nodal_kinematics_batch(const TileDesc* td, int ntiles, int k, int ctas, cudaStream_t s) {
    if (ctas == 2) {
        prefer_shared(k_nodal_kinematics_batch<REINIT, 2>);
        k_nodal_kinematics_batch<REINIT, 2><<<ntiles, TILE_THREADS, 0, s>>>(td, k);
        return;
    }
    prefer_shared(k_nodal_kinematics_batch<REINIT>);
    k_nodal_kinematics_batch<REINIT><<<ntiles, TILE_THREADS, 0, s>>>(td, k);
}

cudaError_t launch_nodal_kinematics_batch(const StepConfig& c, const TileDesc* td, int ntiles,
                                          int k, cudaStream_t s) {
    if (c.reinit) nodal_kinematics_batch<true>(td, ntiles, k, c.nk_ctas, s);
    else nodal_kinematics_batch<false>(td, ntiles, k, c.nk_ctas, s);
    return cudaGetLastError();
}

template <bool USL, bool REINIT, bool TRAC, int MODE>
static void forces_batch_mode(const TileDesc* td, int ntiles, int k, cudaStream_t s) {
    prefer_shared(k_forces_batch<USL, REINIT, TRAC, MODE>);
    k_forces_batch<USL, REINIT, TRAC, MODE><<<ntiles, TILE_THREADS, 0, s>>>(td, k);
}

template <bool USL, bool REINIT, bool TRAC>
static void forces_batch(int mode, const TileDesc* td, int ntiles, int k, cudaStream_t s) {
    if (mode == FM_STAGED) forces_batch_mode<USL, REINIT, TRAC, FM_STAGED>(td, ntiles, k, s);
    else if (mode == FM_LPC) forces_batch_mode<USL, REINIT, TRAC, FM_LPC>(td, ntiles, k, s);
    else forces_batch_mode<USL, REINIT, TRAC, FM_ROW>(td, ntiles, k, s);
}

cudaError_t launch_forces_batch(const StepConfig& c, const TileDesc* td, int ntiles, int k,
                                cudaStream_t s) {
    const int key = (c.usl ? 4 : 0) | (c.reinit ? 2 : 0) | (c.traction ? 1 : 0);
    const int lpc = c.forces_lpc;
    switch (key) {
        case 0: forces_batch<false, false, false>(lpc, td, ntiles, k, s); break;
        case 1: forces_batch<false, false, true>(lpc, td, ntiles, k, s); break;
        case 2: forces_batch<false, true, false>(lpc, td, ntiles, k, s); break;
        case 3: forces_batch<false, true, true>(lpc, td, ntiles, k, s); break;
        case 4: forces_batch<true, false, false>(lpc, td, ntiles, k, s); break;
        case 5: forces_batch<true, false, true>(lpc, td, ntiles, k, s); break;
        case 6: forces_batch<true, true, false>(lpc, td, ntiles, k, s); break;
        default: forces_batch<true, true, true>(lpc, td, ntiles, k, s); break;
    }
    return cudaGetLastError();
}

template <bool USL, bool REINIT>
static void particle_kinematics_batch(const TileDesc* td, int ntiles, int k, int ctas, cudaStream_t s) {
    if (!USL && ctas == 2) {
        prefer_shared(k_particle_kinematics_batch<USL, REINIT, 2>);
        k_particle_kinematics_batch<USL, REINIT, 2><<<ntiles, TILE_THREADS, 0, s>>>(td, k);
        return;
    }
    prefer_shared(k_particle_kinematics_batch<USL, REINIT>);
    k_particle_kinematics_batch<USL, REINIT><<<ntiles, TILE_THREADS, 0, s>>>(td, k);
}

cudaError_t launch_particle_kinematics_batch(const StepConfig& c, const TileDesc* td, int ntiles,
                                             int k, cudaStream_t s) {
    if (c.usl) {
        if (c.reinit) particle_kinematics_batch<true, true>(td, ntiles, k, c.g2p_ctas, s);
        else particle_kinematics_batch<true, false>(td, ntiles, k, c.g2p_ctas, s);
    } else {
        if (c.reinit) particle_kinematics_batch<false, true>(td, ntiles, k, c.g2p_ctas, s);
        else particle_kinematics_batch<false, false>(td, ntiles, k, c.g2p_ctas, s);
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

// ---------------------------------------------------------------------------
// Tile classification.  A tile whose cells and the ring of sort-cells around
// them store no particle receives none during a step block (a particle is at
// most one cell from its sort-cell, and the sort changes only between
// blocks), so its step is a node update only.  At the start of every launched
// sequence the tiles are split into an active list (the step kernels' grid;
// the rest of the grid returns at once) and an empty list (k_empty_nodes),
// each in tile order and padded to ntiles entries with (-1, 0, 0, 0).
// ---------------------------------------------------------------------------
__global__ void k_tile_flags(const __grid_constant__ SimDev S, const int4* __restrict__ tiles, int ntiles,
                             int* __restrict__ flags) {
    const int t = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31;
    if (t >= ntiles) return;
    const int4 T = tiles[t];
    const int c0x = T.y * TILE_NX - 1, c0y = T.z * TILE_NY - 1;
    const int x0 = max(c0x - 1, 0), x1 = min(c0x + TILE_CX + 1, S.nx);
    const int y0 = max(c0y - 1, 0), y1 = min(c0y + TILE_CY + 1, S.ny);
    int occ = 0;
    if (x0 < x1)
        for (int r = y0 + lane; r < y1; r += 32) occ |= S.cstart[r * S.nx + x1] != S.cstart[r * S.nx + x0];
    occ = __any_sync(0xffffffffu, occ);
    if (lane == 0) flags[t] = occ;
}

__global__ void __launch_bounds__(1024)
k_compact_tiles(const int* __restrict__ flags, const int4* __restrict__ tiles, int ntiles,
                int4* __restrict__ active, int4* __restrict__ empty, int* __restrict__ counts) {
    __shared__ int base[2];
    if (threadIdx.x == 0) base[0] = base[1] = 0;
    __syncthreads();
    for (int c = 0; c < ntiles; c += 1024) {
        const int t = c + (int)threadIdx.x;
        const int f = t < ntiles ? (flags[t] != 0) : 0;
        const int g = t < ntiles ? 1 - f : 0;
        int tot_a, tot_e;
        const int pa = block_exclusive_scan(f, &tot_a);
        const int pe = block_exclusive_scan(g, &tot_e);
        if (t < ntiles) {
            if (f) active[base[0] + pa] = tiles[t];
            else empty[base[1] + pe] = tiles[t];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            base[0] += tot_a;
            base[1] += tot_e;
        }
        __syncthreads();
    }
    const int4 none = make_int4(-1, 0, 0, 0);
    for (int i = base[0] + (int)threadIdx.x; i < ntiles; i += 1024) active[i] = none;
    for (int i = base[1] + (int)threadIdx.x; i < ntiles; i += 1024) empty[i] = none;
    if (threadIdx.x == 0 && counts) {
        counts[0] = base[0];
        counts[1] = base[1];
    }
}

cudaError_t launch_classify_tiles(const SimDev& S, const int4* tiles, int ntiles, int* flags, int4* active,
                                  int4* empty, int* counts, cudaStream_t s) {
    if (ntiles > 0) {
        k_tile_flags<<<(ntiles + 7) / 8, 256, 0, s>>>(S, tiles, ntiles, flags);
        k_compact_tiles<<<1, 1024, 0, s>>>(flags, tiles, ntiles, active, empty, counts);
    }
    return cudaGetLastError();
}

// The step of the nodes of an empty tile: the nodal kinematics of a massless
// node (nodal_kinematics_tile's empty path) and the nodal update with no
// particle force (forces_tile's empty path), in one pass.  It runs before
// the step's nodal-kinematics launch: no other tile reads these nodes' values
// until the forces kernel (their velocity after nodal kinematics) and G2P
// (their updated velocity and acceleration).  A CTA covers EMPTY_TILES tiles,
// thread (lx, ly) the node (lx, ly) of each, with all loads of its nodes in
// flight together: the kernel is a few loads and stores per node, so it is
// latency that bounds it.
constexpr int EMPTY_TILES = 4;

__device__ __forceinline__ void empty_node_step(const SimDev& S, int node, uint16_t ncons, float vbx,
                                                float vby, float t) {
    float vx = flush(vbx), vy = flush(vby);
    apply_constraint(S, ncons, vx, vy, nullptr, nullptr);
    S.nm[node] = 0.0f;
    S.nvax[node] = vx;
    S.nvay[node] = vy;
    nodal_update<false, true>(S, node, t, 0.0f, 0.0f, vx, vy, 0.0f, ncons);
}

__global__ void __launch_bounds__(TILE_THREADS)
k_empty_nodes(const __grid_constant__ SimDev S, const int4* __restrict__ empty, int nempty,
              Control* __restrict__ ctl, int k) {
    const int tid = threadIdx.x, lx = tid & (TILE_CX - 1), ly = tid / TILE_CX;
    const float t = step_time(load_step(ctl) + k, S.dt);
    int node[EMPTY_TILES];
    uint16_t nc[EMPTY_TILES];
    float vbx[EMPTY_TILES], vby[EMPTY_TILES];
    #pragma unroll
    for (int e = 0; e < EMPTY_TILES; ++e) {
        const int slot = blockIdx.x * EMPTY_TILES + e;
        node[e] = -1;
        if (slot < nempty) {
            const int4 T = empty[slot];
            const int c0x = T.y * TILE_NX - 1, c0y = T.z * TILE_NY - 1;
            if (T.x >= 0 && lx < TILE_NX && ly < TILE_NY && c0x + 1 + lx <= S.nx && c0y + 1 + ly <= S.ny)
                node[e] = (c0y + 1 + ly) * (S.nx + 1) + c0x + 1 + lx;
        }
    }
    #pragma unroll
    for (int e = 0; e < EMPTY_TILES; ++e)
        if (node[e] >= 0) {
            nc[e] = S.ncons[node[e]];
            vbx[e] = S.nvbx[node[e]];
            vby[e] = S.nvby[node[e]];
        }
    #pragma unroll
    for (int e = 0; e < EMPTY_TILES; ++e)
        if (node[e] >= 0) empty_node_step(S, node[e], nc[e], vbx[e], vby[e], t);
}

cudaError_t launch_empty_nodes(const SimDev& S, const int4* empty, int ntiles, Control* ctl, int k,
                               cudaStream_t s) {
    if (ntiles > 0)
        k_empty_nodes<<<(ntiles + EMPTY_TILES - 1) / EMPTY_TILES, TILE_THREADS, 0, s>>>(S, empty, ntiles, ctl,
                                                                                       k);
    return cudaGetLastError();
}

// The same split for the tiles of a batch (each tile's simulation from sims).
__global__ void k_tile_flags_batch(const SimDev* const* __restrict__ sims, const int4* __restrict__ tiles,
                                   int ntiles, int* __restrict__ flags) {
    const int t = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31;
    if (t >= ntiles) return;
    const int4 T = tiles[t];
    const SimDev* S = sims[T.x];
    const int nx = S->nx, ny = S->ny;
    const int* __restrict__ cstart = S->cstart;
    const int c0x = T.y * TILE_NX - 1, c0y = T.z * TILE_NY - 1;
    const int x0 = max(c0x - 1, 0), x1 = min(c0x + TILE_CX + 1, nx);
    const int y0 = max(c0y - 1, 0), y1 = min(c0y + TILE_CY + 1, ny);
    int occ = 0;
    if (x0 < x1)
        for (int r = y0 + lane; r < y1; r += 32) occ |= cstart[r * nx + x1] != cstart[r * nx + x0];
    occ = __any_sync(0xffffffffu, occ);
    if (lane == 0) flags[t] = occ;
}

cudaError_t launch_classify_tiles_batch(const SimDev* const* sims, const int4* tiles, int ntiles, int* flags,
                                        int4* active, int4* empty, int* counts, cudaStream_t s) {
    if (ntiles > 0) {
        k_tile_flags_batch<<<(ntiles + 7) / 8, 256, 0, s>>>(sims, tiles, ntiles, flags);
        k_compact_tiles<<<1, 1024, 0, s>>>(flags, tiles, ntiles, active, empty, counts);
    }
    return cudaGetLastError();
}

// k_empty_nodes for the empty tiles of a batch, from their tile records (the
// record's head: tile, control pointer and descriptor), EMPTY_TILES tiles per
// CTA.
__global__ void __launch_bounds__(TILE_THREADS)
k_empty_nodes_batch(const TileDesc* __restrict__ td, int nempty, int k) {
    constexpr int HEAD = (int)((offsetof(TileDesc, occ) + 15) / 16);   // tile, control, descriptor
    __shared__ int4 s_head[EMPTY_TILES][HEAD];
    const int first = blockIdx.x * EMPTY_TILES;
    for (int i = threadIdx.x; i < EMPTY_TILES * HEAD; i += blockDim.x) {
        const int e = i / HEAD, w = i - e * HEAD;
        if (first + e < nempty) s_head[e][w] = reinterpret_cast<const int4*>(td + first + e)[w];
    }
    __syncthreads();
    const int tid = threadIdx.x, lx = tid & (TILE_CX - 1), ly = tid / TILE_CX;
    int node[EMPTY_TILES];
    uint16_t nc[EMPTY_TILES];
    float vbx[EMPTY_TILES], vby[EMPTY_TILES];
    #pragma unroll
    for (int e = 0; e < EMPTY_TILES; ++e) {
        node[e] = -1;
        if (first + e < nempty) {
            const TileDesc& R = *reinterpret_cast<const TileDesc*>(s_head[e]);
            const int4 T = R.T;
            const int c0x = T.y * TILE_NX - 1, c0y = T.z * TILE_NY - 1;
            if (T.x >= 0 && lx < TILE_NX && ly < TILE_NY && c0x + 1 + lx <= R.S.nx && c0y + 1 + ly <= R.S.ny)
                node[e] = (c0y + 1 + ly) * (R.S.nx + 1) + c0x + 1 + lx;
        }
    }
    #pragma unroll
    for (int e = 0; e < EMPTY_TILES; ++e)
        if (node[e] >= 0) {
            const SimDev& S = reinterpret_cast<const TileDesc*>(s_head[e])->S;
            nc[e] = S.ncons[node[e]];
            vbx[e] = S.nvbx[node[e]];
            vby[e] = S.nvby[node[e]];
        }
    #pragma unroll
    for (int e = 0; e < EMPTY_TILES; ++e)
        if (node[e] >= 0) {
            const TileDesc& R = *reinterpret_cast<const TileDesc*>(s_head[e]);
            empty_node_step(R.S, node[e], nc[e], vbx[e], vby[e], step_time(load_step(R.ctl) + k, R.S.dt));
        }
}

cudaError_t launch_empty_nodes_batch(const TileDesc* td, int ntiles, int k, cudaStream_t s) {
    if (ntiles > 0)
        k_empty_nodes_batch<<<(ntiles + EMPTY_TILES - 1) / EMPTY_TILES, TILE_THREADS, 0, s>>>(td, ntiles, k);
    return cudaGetLastError();
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

// what: 0 element id (int32), 1 volume, 2 mass, 3 momentum (ndim comps)
__global__ void k_derived_out(const SimDev* __restrict__ sim, int ndim, int np, int parity, int reinit,
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
        // element volume: the 2-D formula, or the element length in 1-D
        const float vel = ndim == 1 ? fs(node_coord(i + 1, S.hx), node_coord(i, S.hx)) : S.vol_el;
        V = cnt ? fdv(vel, (float)cnt) : 0.0f;
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
    } else if (ndim == 1) {
        static_cast<float*>(out)[o] = fm(m, S.vx[q]);
    } else {
        static_cast<float*>(out)[2 * (size_t)o] = fm(m, S.vx[q]);
        static_cast<float*>(out)[2 * (size_t)o + 1] = fm(m, S.vy[q]);
    }
}

cudaError_t launch_derived_out(const SimDev* sim, int ndim, int np, int parity, bool reinit, int what,
                               const int* pid, void* out, cudaStream_t s) {
    if (np > 0)
        k_derived_out<<<(np + 255) / 256, 256, 0, s>>>(sim, ndim, np, parity, reinit ? 1 : 0, what, pid, out);
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
    if (i < n && !vy) {
        out[i] = fm(m[i], vx[i]);   // 1-D
    } else if (i < n) {
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

// ---------------------------------------------------------------------------
// Segmented copy and status gather for batches
// ---------------------------------------------------------------------------
// Chunk table: chunk b of segment i (the last i with first[i] <= b).
__global__ void k_chunk_table(const CopySeg* __restrict__ segs, const unsigned* __restrict__ first,
                              int nseg, unsigned nchunks, CopyChunk* __restrict__ chunks) {
    const unsigned b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nchunks) return;
    int lo = 0, hi = nseg - 1;
    #pragma unroll 1
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (first[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    const CopySeg sg = segs[lo];
    const unsigned long long off = (unsigned long long)(b - first[lo]) * COPY_CHUNK;
    CopyChunk c;
    c.src = static_cast<const char*>(sg.src) + off;
    c.dst = static_cast<char*>(sg.dst) + off;
    c.dst_step = sg.dst_step;
    c.bytes = off < sg.bytes ? min((unsigned long long)COPY_CHUNK, sg.bytes - off) : 0ull;
    chunks[b] = c;
}

cudaError_t launch_chunk_table(const CopySeg* segs, const unsigned* first, int nseg, unsigned nchunks,
                               CopyChunk* chunks, cudaStream_t s) {
    if (nseg > 0 && nchunks > 0)
        k_chunk_table<<<(nchunks + 255) / 256, 256, 0, s>>>(segs, first, nseg, nchunks, chunks);
    return cudaGetLastError();
}

// A CTA of COPY_THREADS threads moves one chunk as COPY_VEC 16-byte words a
// thread, all loaded before any is stored.  The destinations (tape slots,
// checkpoints, snapshots) are not read again soon: streaming stores.
constexpr int COPY_THREADS = 256;
constexpr int COPY_VEC = COPY_CHUNK / (16 * COPY_THREADS);
static_assert(COPY_VEC * 16 * COPY_THREADS == COPY_CHUNK, "a chunk is whole words of every thread");

__device__ __forceinline__ CopyChunk load_chunk(const CopyChunk* __restrict__ chunks, unsigned b) {
    const ulonglong2* p = reinterpret_cast<const ulonglong2*>(chunks + b);
    const ulonglong2 u = p[0], w = p[1];
    CopyChunk c;
    c.src = reinterpret_cast<const char*>(u.x);
    c.dst = reinterpret_cast<char*>(u.y);
    c.dst_step = w.x;
    c.bytes = w.y;
    return c;
}

__global__ void __launch_bounds__(COPY_THREADS)
k_copy_segments(const CopyChunk* __restrict__ chunks, int t) {
    static_assert(sizeof(CopyChunk) == 32, "chunk entries are read as two 16-byte words");
    const CopyChunk c = load_chunk(chunks, blockIdx.x);
    const char* __restrict__ src = c.src;
    char* __restrict__ dst = c.dst + (unsigned long long)t * c.dst_step;
    const unsigned n = (unsigned)c.bytes;
    const bool vec = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15) == 0;
    const unsigned n16 = vec ? n >> 4 : 0;
    const uint4* __restrict__ s4 = reinterpret_cast<const uint4*>(src);
    uint4* __restrict__ d4 = reinterpret_cast<uint4*>(dst);
    uint4 v[COPY_VEC];
    #pragma unroll
    for (int u = 0; u < COPY_VEC; ++u) {
        const unsigned k = threadIdx.x + u * COPY_THREADS;
        if (k < n16) v[u] = s4[k];
    }
    #pragma unroll
    for (int u = 0; u < COPY_VEC; ++u) {
        const unsigned k = threadIdx.x + u * COPY_THREADS;
        if (k < n16) __stcs(d4 + k, v[u]);
    }
    for (unsigned k = 16 * n16 + threadIdx.x; k < n; k += COPY_THREADS) dst[k] = src[k];
}

cudaError_t launch_copy_segments(const CopyChunk* chunks, unsigned nchunks, int t, cudaStream_t s) {
    if (nchunks > 0) k_copy_segments<<<nchunks, COPY_THREADS, 0, s>>>(chunks, t);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(COPY_THREADS)
k_compare_segments(const CopyChunk* __restrict__ chunks, int* __restrict__ mismatch) {
    const CopyChunk c = load_chunk(chunks, blockIdx.x);
    const char* a = c.src;
    const char* d = c.dst;
    const unsigned n = (unsigned)c.bytes;
    const bool vec = ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(d)) & 15) == 0;
    const unsigned n16 = vec ? n >> 4 : 0;
    int diff = 0;
    const uint4* a4 = reinterpret_cast<const uint4*>(a);
    const uint4* d4 = reinterpret_cast<const uint4*>(d);
    #pragma unroll
    for (int u = 0; u < COPY_VEC; ++u) {
        const unsigned k = threadIdx.x + u * COPY_THREADS;
        if (k < n16) {
            const uint4 x = a4[k], y = d4[k];
            diff += (x.x != y.x) | (x.y != y.y) | (x.z != y.z) | (x.w != y.w);
        }
    }
    for (unsigned k = 16 * n16 + threadIdx.x; k < n; k += COPY_THREADS) diff += a[k] != d[k];
    const int total = __syncthreads_count(diff != 0);
    if (threadIdx.x == 0 && total) atomicAdd(mismatch, total);
}

cudaError_t launch_compare_segments(const CopyChunk* chunks, unsigned nchunks, int* mismatch,
                                    cudaStream_t s) {
    if (nchunks > 0) k_compare_segments<<<nchunks, COPY_THREADS, 0, s>>>(chunks, mismatch);
    return cudaGetLastError();
}

__global__ void k_gather_status(Control* const* __restrict__ ctls, int n, Control* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Control* c = ctls[i];
    out[i] = *c;
    c->status = 0;
}

cudaError_t launch_gather_status(Control* const* ctls, int n, Control* out, cudaStream_t s) {
    if (n > 0) k_gather_status<<<(n + 127) / 128, 128, 0, s>>>(ctls, n, out);
    return cudaGetLastError();
}

}  // namespace mpm
