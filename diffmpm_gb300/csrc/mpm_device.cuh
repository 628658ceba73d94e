// Device helpers of the explicit MPM step.
//
// Every floating-point operation that the reference performs is written with
// an explicitly rounded intrinsic (__fmul_rn, __fadd_rn, ...) in the order the
// reference writes it, so no multiply-add is ever fused and the per-particle
// arithmetic is reproducible operation by operation.
#pragma once
#include <cfloat>
#include <cstdint>
#include "mpm_types.h"

namespace mpm {

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fdv(float a, float b) { return __fdiv_rn(a, b); }

// Asynchronous 4-byte global -> shared copies (cp.async), committed in groups.
__device__ __forceinline__ void cp_async4(void* smem_dst, const void* gmem_src) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(smem_dst));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(gmem_src) : "memory");
}
// 16-byte global -> shared copy through L2 only (cp.async.cg); both
// addresses 16-byte aligned.
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gmem_src) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(smem_dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// where(|a| < 1e-12, 0, a) (diffmpm/element.py:185-189, particle.py:310-312)
__device__ __forceinline__ float flush(float a) { return fabsf(a) < 1e-12f ? 0.0f : a; }

// jnp.nan_to_num: NaN -> 0, +/-inf -> +/-FLT_MAX (diffmpm/element.py:311)
__device__ __forceinline__ float nan_to_num(float a) {
    if (isnan(a)) return 0.0f;
    if (isinf(a)) return a > 0.0f ? FLT_MAX : -FLT_MAX;
    return a;
}

// Node coordinate i*h as the reference forms it: float(i) * h rounded once
// (diffmpm/element.py:669-679).
__device__ __forceinline__ float node_coord(int i, float h) { return fm((float)i, h); }

// Largest i in [0, n] with node_coord(i) <= x, or -1 (none, or x is NaN).
// Same ids as diffmpm/element.py:820-840 for particles strictly inside.
__device__ __forceinline__ int locate_axis(float x, float h, int n) {
    float q = fdv(x, h);
    int i;
    if (!(q >= -1.0f)) {
        i = -1;
    } else if (q >= (float)n + 1.0f) {
        i = n;
    } else {
        i = (int)floorf(q);
    }
    #pragma unroll 1
    for (int it = 0; it < 4 && i < n && node_coord(i + 1, h) <= x; ++it) ++i;
    #pragma unroll 1
    for (int it = 0; it < 4 && i >= 0 && node_coord(i, h) > x; ++it) --i;
    return i;
}

// Geometry of cell (i, j): bounds, centre and 2/width (diffmpm/particle.py:202-205;
// the same factor is the inverse Jacobian of the axis-aligned element).
struct CellGeo {
    float x0, x1, y0, y1;
    float cx, cy;   // (x0 + x1) / 2
    float rx, ry;   // 2 / (x1 - x0)
};

__device__ __forceinline__ CellGeo cell_geo(int i, int j, float hx, float hy) {
    CellGeo g;
    g.x0 = node_coord(i, hx);
    g.x1 = node_coord(i + 1, hx);
    g.y0 = node_coord(j, hy);
    g.y1 = node_coord(j + 1, hy);
    g.cx = fm(fa(g.x0, g.x1), 0.5f);
    g.cy = fm(fa(g.y0, g.y1), 0.5f);
    g.rx = fdv(2.0f, fs(g.x1, g.x0));
    g.ry = fdv(2.0f, fs(g.y1, g.y0));
    return g;
}

__device__ __forceinline__ bool in_cell(const CellGeo& g, float x, float y) {
    return g.x0 <= x && x < g.x1 && g.y0 <= y && y < g.y1;
}

// Natural coordinate (x - (x0+x1)/2) * (2/(x1-x0)) (diffmpm/particle.py:203-205).
__device__ __forceinline__ float natural(float x, float c, float r) { return fm(fs(x, c), r); }

// Q4 shape functions in node order 0..3 (diffmpm/element.py:748-757).
__device__ __forceinline__ void shape4(float xi, float eta, float N[4]) {
    const float a = fs(1.0f, xi), b = fa(1.0f, xi), c = fs(1.0f, eta), d = fa(1.0f, eta);
    N[0] = fm(fm(0.25f, a), c);
    N[1] = fm(fm(0.25f, b), c);
    N[2] = fm(fm(0.25f, b), d);
    N[3] = fm(fm(0.25f, a), d);
}

// dN/dx, dN/dy: natural gradient (diffmpm/element.py:781-788) times the
// inverse Jacobian diag(rx, ry) of the axis-aligned element (element.py:814-817).
// Rounding to nearest is symmetric in sign, so (-0.25 c) rx is exactly
// -((0.25 c) rx): each pair of opposite entries costs one product, and the
// products 0.25 a, 0.25 b are those of shape4.
__device__ __forceinline__ void dshape4(float xi, float eta, float rx, float ry,
                                        float Gx[4], float Gy[4]) {
    const float a = fs(1.0f, xi), b = fa(1.0f, xi), c = fs(1.0f, eta), d = fa(1.0f, eta);
    const float gc = fm(fm(0.25f, c), rx), gd = fm(fm(0.25f, d), rx);
    const float ga = fm(fm(0.25f, a), ry), gb = fm(fm(0.25f, b), ry);
    Gx[0] = -gc;
    Gx[1] = gc;
    Gx[2] = gd;
    Gx[3] = -gd;
    Gy[0] = -ga;
    Gy[1] = -gb;
    Gy[2] = gb;
    Gy[3] = ga;
}

// sum_k A[k] * B[k], left to right.
__device__ __forceinline__ float dot4(const float A[4], const float B[4]) {
    float s = fm(A[0], B[0]);
    s = fa(s, fm(A[1], B[1]));
    s = fa(s, fm(A[2], B[2]));
    s = fa(s, fm(A[3], B[3]));
    return s;
}

// Strain rate [M00, M11, M01 + M10] with M = dN/dx^T v, flushed
// (diffmpm/particle.py:281-313).
__device__ __forceinline__ void strain_rate4(const float Gx[4], const float Gy[4],
                                             const float vx[4], const float vy[4],
                                             float& r0, float& r1, float& r3) {
    r0 = flush(dot4(Gx, vx));
    r1 = flush(dot4(Gy, vy));
    r3 = flush(fa(dot4(Gx, vy), dot4(Gy, vx)));
}

// Piecewise-linear time function (diffmpm/functions.py:40-41, jnp.interp);
// code 1 = Unit (functions.py:24-25), k + 2 = table k.
template <class Tables>   // SimDev, or any struct with the same fn_off, fn_x, fn_y
__device__ __forceinline__ float fn_value(const Tables& S, int code, float t) {
    if (code <= 1) return 1.0f;
    const int k = code - 2;
    const int b = S.fn_off[k], n = S.fn_off[k + 1] - b;
    const float* X = S.fn_x + b;
    const float* Y = S.fn_y + b;
    if (n <= 1) return Y[0];
    if (t < X[0]) return Y[0];
    if (t > X[n - 1]) return Y[n - 1];
    int i = 1;
    #pragma unroll 1
    while (i < n - 1 && X[i] <= t) ++i;
    const float dx = fs(X[i], X[i - 1]);
    if (fabsf(dx) <= 1.4210855e-14f) return Y[i - 1];
    return fa(Y[i - 1], fm(fdv(fs(t, X[i - 1]), dx), fs(Y[i], Y[i - 1])));
}

// Current time t = float(i) * dt (diffmpm/scheme.py:52-54).
__device__ __forceinline__ float step_time(int step, float dt) { return fm((float)step, dt); }

// Particle state touched by the strain/stress update.
struct PState {
    float sxx, syy, szz, sxy;
    float exx, eyy, exy;
    float rho, vsc;
};

// compute_strain + update_volume + compute_stress for one particle
// (diffmpm/particle.py:249-327, material.py:113-131).  `Ep` is the per-particle
// Young's modulus (LinearElastic) or a negative value for the material's own.
// Returns the volume factor 1 + dvol.
__device__ __forceinline__ float strain_stress_update(const MatDev& M, float Ep, float dt,
                                                      float r0, float r1, float r3,
                                                      float dvol, PState& p) {
    const float d0 = fm(r0, dt), d1 = fm(r1, dt), d3 = fm(r3, dt);
    p.exx = fa(p.exx, d0);
    p.eyy = fa(p.eyy, d1);
    p.exy = fa(p.exy, d3);
    p.vsc = fa(p.vsc, dvol);
    const float f = fa(1.0f, dvol);
    p.rho = fdv(p.rho, f);
    if (M.type == MAT_LINEAR_ELASTIC) {
        float a1 = M.a1, a2 = M.a2, G = M.G;
        if (Ep >= 0.0f) {
            a1 = fm(Ep, M.c1);
            a2 = fm(Ep, M.c2);
            G = fm(Ep, M.c3);
        }
        p.sxx = fa(p.sxx, fa(fm(a1, d0), fm(a2, d1)));
        p.syy = fa(p.syy, fa(fm(a2, d0), fm(a1, d1)));
        p.szz = fa(p.szz, fa(fm(a2, d0), fm(a2, d1)));
        p.sxy = fa(p.sxy, fm(G, d3));
    } else if (M.type == MAT_SIMPLE) {
        const float E = Ep >= 0.0f ? Ep : M.E;   // a per-particle E replaces the material's
        p.sxx = fa(p.sxx, fm(d0, E));
        p.syy = fa(p.syy, fm(d1, E));
        p.sxy = fa(p.sxy, fm(d3, E));
    } else {
        // Newtonian (build definition): total stress from the strain rate and
        // the centroid volumetric strain, p = -K * vsc.
        const float kv = fm(M.K, p.vsc);
        const float t3 = fdv(fa(r0, r1), 3.0f);
        p.sxx = fa(kv, fm(M.twomu, fs(r0, t3)));
        p.syy = fa(kv, fm(M.twomu, fs(r1, t3)));
        p.szz = fs(kv, fm(M.twomu, t3));
        p.sxy = fm(M.mu, r3);
    }
    return f;
}

// ---------------------------------------------------------------------------
// Tile helpers shared by the forward and reverse kernels: a CTA of
// TILE_THREADS threads covers TILE_CX x TILE_CY cells, thread tid = cell
// (tid % TILE_CX, tid / TILE_CX), and owns the node at the upper-right corner
// of its cell for lx < TILE_NX, ly < TILE_NY.
// ---------------------------------------------------------------------------
// Sum of the four cell-corner partials meeting at the node of thread `tid`
// (node = lower-left corner of cell tid + 33): cell (I-1,J-1) corner 2,
// cell (I,J-1) corner 3, cell (I-1,J) corner 1, cell (I,J) corner 0.
constexpr int SC_STRIDE = TILE_THREADS + 1;   // per-quantity row of the cell-corner partials

__device__ __forceinline__ float node_sum(const float (*s)[SC_STRIDE], int tid) {
    return fa(fa(fa(s[2][tid], s[3][tid + 1]), s[1][tid + TILE_CX]), s[0][tid + TILE_CX + 1]);
}

// Fast path of the particle-to-grid gathers (forward and reverse): warp w
// stages the particles stored in sort-cell row w of a tile (storage range
// [rb, re)) into shared memory with coalesced copies, and lane l then visits
// the particles of its own cell (storage range [cb, ce)) in storage order,
// summing their corner contributions in registers: the same order and the
// same roundings as the slow path's visit_cell, so both paths give the same
// bits.  Pass k stages storage slots [rb4 + kP, rb4 + (k+1)P) (rb4 = rb
// rounded down to a multiple of 4, P a multiple of 4) of every field with
// one cp.async.cg per 16-byte piece, and f(q, j) finds slot q at buf[.][j],
// j = q - (rb4 + kP).  Every source array must start on a 16-byte boundary
// and hold a multiple of 4 slots (the last piece may read up to 3 slots past
// re).
template <int NF, int P, class F>
__device__ __forceinline__ void row_pass16(float (*buf)[P], const float* const (&src)[NF], int rb,
                                           int re, int cb, int ce, int lane, F&& f) {
    static_assert(P % 4 == 0, "passes start on 16-byte boundaries");
    #pragma unroll 1
    for (int p0 = rb & ~3; p0 < re; p0 += P) {
        const int p1 = min(p0 + P, re);
        #pragma unroll
        for (int k = 0; k < NF; ++k) {
            if (!src[k]) continue;
            #pragma unroll
            for (int o = 4 * lane; o < P; o += 128)
                if (p0 + o < p1) cp_async16(&buf[k][o], src[k] + p0 + o);
        }
        cp_async_commit();
        cp_async_wait<0>();
        __syncwarp();
        const int lo = max(cb, p0), hi = min(ce, p1);
        #pragma unroll 1
        for (int q = lo; q < hi; ++q) f(q, q - p0);
        __syncwarp();
    }
}

}  // namespace mpm
