// Device-visible simulation descriptor shared by the kernels and the host driver.
//
// Layout in HBM (one simulation; a batch is an array of these):
//   particles  SoA float32 in cell-sorted storage order.  Fields that a tile
//              reads for its one-cell halo while the owner tile rewrites them
//              (stress, density, volumetric strain, volume) are ping-pong
//              pairs indexed by the step parity; the rest are single arrays.
//   cells      cstart[Ne+1]: storage range of each sort-cell (cell at the last
//              re-sort); cflag[Ne]: 1 when a particle stored in the sort-cell
//              is currently in another cell.
//   nodes      mass, velocity after the nodal-kinematics phase (nva*),
//              velocity and acceleration after the nodal update (nvb*, na*),
//              a 16-bit constraint code per node.
#pragma once
#include <stdint.h>

namespace mpm {

constexpr int TILE_CX = 32;              // cells per tile row (one warp)
constexpr int TILE_CY = 16;              // cell rows per tile
constexpr int TILE_NX = TILE_CX - 1;     // nodes owned per tile row
constexpr int TILE_NY = TILE_CY - 1;     // node rows owned per tile
constexpr int TILE_THREADS = TILE_CX * TILE_CY;
constexpr int TILE_MIN_CTAS = 16 / TILE_CY * 2;   // resident CTAs per SM the kernels are built for
// The nodal kinematics and USF G2P kernels fit 40 registers a thread and
// < 75 KB of shared memory, so three of their CTAs are resident per SM.
constexpr int TILE_CTAS_LIGHT = 3 * TILE_MIN_CTAS / 2;

enum StatusBits : int {
    ST_OUT_OF_MESH = 1,     // a particle left the mesh
    ST_DRIFT_VIOLATION = 2, // a particle is more than one cell from its sort-cell
    ST_DRIFTED = 4,         // some particle is in a cell other than its sort-cell
    ST_TRACTION_CONFLICT = 8
};

enum MatType : int { MAT_LINEAR_ELASTIC = 0, MAT_SIMPLE = 1, MAT_NEWTONIAN = 2 };

struct MatDev {
    int type;
    float a1, a2, G;       // LinearElastic D-matrix entries (host float64 -> float32)
    float c1, c2, c3;      // a1, a2, G per unit Young's modulus (per-particle E)
    float E;               // SimpleMaterial
    float K, mu, twomu;    // Newtonian
    float density;
};

struct SimDev {
    // mesh
    int nx, ny;
    float hx, hy;
    float vol_el;          // element volume (reference formula, float32)
    float dt;
    float gx, gy;
    int tiles_x, tiles_y;
    int np;
    int velocity_update;
    // particles (storage order)
    float *x, *y, *vx, *vy;
    float *sxx[2], *syy[2], *szz[2], *sxy[2];
    float *exx, *eyy, *exy;
    float *rho[2], *vsc[2];
    float *vol[2];         // persistent volume (solve semantics only)
    float *mass;           // persistent mass (solve semantics only)
    float *psize;          // persistent size (solve semantics with tractions only)
    uint8_t *mat;
    float *E;              // per-particle Young's modulus or null
    int8_t *tr_fn;         // [2 per particle] 0 none, 1 Unit, k+2 table k; null if no tractions
    float *tr_tau;         // [2 per particle]
    int *pid;              // storage index -> original particle index
    const uint8_t *pvc;    // [2 per particle] velocity constraint slot+1 per direction, or null
    const float *pvc_vel;  // particle velocity constraint table
    // cells
    int *cstart;
    uint8_t *cflag;
    // nodes
    float *nm;
    float *nvax, *nvay;
    float *nvbx, *nvby;
    float *nax, *nay;
    uint16_t *ncons;       // low byte: dir-0 velocity slot+1, high byte: dir-1 slot+1
    const float *cons_vel; // constraint velocity table
    const int *cnf_ptr;    // CSR per node into the nodal-force entries (null if none)
    const int8_t *cnf_dir;
    const float *cnf_val;
    const int8_t *cnf_fn;  // 1 Unit, k+2 table k
    // time functions
    int nfn;
    const int *fn_off;     // nfn+1 offsets
    const float *fn_x, *fn_y;
    // materials
    int nmat;
    const MatDev *mats;
};

struct Control;

// One tile of a batched launch together with its simulation's descriptor and
// control block, so that a CTA fetches everything it needs to start in one
// contiguous read (refreshed before every step block).  The storage starts
// of the tile's cell rows and whether any particle is stored around the tile
// change only at a re-sort, which happens between step blocks, so they are
// part of the record too: a batched CTA then issues its particle loads right
// after the record arrives, as a single-simulation CTA does after its own
// set-up loads.
struct alignas(16) TileDesc {
    int4 T;                // (simulation, tile x, tile y, 0)
    Control* ctl;
    long long pad;
    SimDev S;
    int occ;               // a particle is stored in sort-cells [c0x-1, c0x+33) x [c0y-1, c0y+17)
    int pad2[3];
    int cs[TILE_CY][33];   // storage start of cell (c0x + l, c0y + r), l clamped to [0, nx]; 0 off the mesh
};
static_assert(sizeof(TileDesc) % 16 == 0, "tile records are copied in 16-byte pieces");

// Per-batch control block.
struct Control {
    int step;              // step counter i (t = i * dt) at the start of the launched sequence
    int status;            // StatusBits
    unsigned int done;     // reserved (zero)
    int pad;
};

}  // namespace mpm
