// Fluid passes on sm_103a, reference precision (FP32 fluid state).
//
//   fluid pair       findFluidPair + fluidFluid/Solid/VirtCalculate
//                    (fluid.cu:25-254): Riemann continuity and momentum,
//                    velocity gradient, colour, kernel-gradient sum and the
//                    near-free-surface flag, summed over the 3x3 stencil in
//                    the reference's list order (fluid, solid, virtual per
//                    neighbour cell, slots 0..8).
//   k_fluid_update   fluidUpdate (fluid.cu:256-287) fused with getMaxSpeed
//                    (fluid.cu:429-440): the max of |v| is reduced on the
//                    device (the reference copies every velocity to the host
//                    each step).  |v|^2 is formed with round-to-nearest
//                    multiplies and adds and compared as float bits, which
//                    equals the reference's host loop over |v| (sqrt is
//                    monotone), so max_speed is bit-identical.
//   shifting pass    correctionCalculate (fluid.cu:304-367) fused with
//                    shiftDisplacementCalculate + correctionUpdate
//                    (fluid.cu:369-427): the thread that sums a particle's
//                    shifting gradient also moves it, into a second position
//                    buffer (the passes alternate between the two)
//
// The two neighbour sweeps are tiled: a block owns a column segment of
// `tile_h` cells and stages the fluid neighbours of that segment - three
// column strips of tile_h + 2 cells, each a contiguous range of the CSR list
// - into shared memory once.  Every thread then walks its own particle's 3x3
// stencil in the reference's order, reading fluid neighbours from shared
// memory (solid and virtual neighbours, rare, from global memory), so the
// per-particle sums are the same sums in the same order as the per-particle
// form.  The shifting passes also stage the tile's virtual strips, so that a
// particle next to a wall walks a stored list like any other.  Particles that are in no cell list (moved more than one cell since
// the last sort) are handled by per-particle fallback kernels, which return
// at once when every particle is listed.
//
// Math: the neighbour sweeps use __expf, __fdividef and sqrt.approx, the
// approximations that the reference's -use_fast_math build uses for expf,
// '/' and sqrtf (CMakeLists.txt:16-19); the equation of state keeps powf,
// whose fast form loses ~1e-4 relative pressure accuracy near the reference
// density.  The mixed form's pair term uses SFU reciprocals (riemann).
#include "forms.cuh"
#include "kernels.h"

#include <algorithm>
#include <cmath>
#include <type_traits>

namespace sphnj {

namespace {

constexpr int kPairBlock = 128;
constexpr int kTileBlock = 256;   // tiled sweeps: ~208 particles per 16-cell tile
constexpr int kListBlock = 128;   // shifting passes over an active-tile list
constexpr int kDenseBlock = 128;  // shifting passes of a dense scene, one block per tile

// Block shape of the pair pass, by launch:
//  - batches (tile lists): 128 threads, 8 blocks per SM (64 registers, no
//    spills), staging sized by pair_per_cell so that the 8 fit.  Smaller
//    blocks leave fewer warps waiting at a tile's barriers (256-scene mixed
//    sweep 4.56 -> 4.46 ms/step);
//  - a dense scene swept alone (one block per tile): 128 threads, 8 per SM
//    in the plain form, 7 in the mixed form.  4.15M dam break 3.80 -> 3.74
//    ms/step at 8 per SM against 256 threads at 5; then, measured on one box,
//    mixed 3.737 at 8 against 3.660 at 7, plain 4.214 at 8 against 4.267 at 7
//    (6 per SM: 3.76);
//  - a sparse scene swept alone (tile list): 256 threads, 5 per SM (48
//    registers; unbounded it takes 64 and 4 blocks).
template <class G, bool kList, class F> struct PairShape {
    static constexpr int threads = 128, min_blocks = 8;
};
template <> struct PairShape<GroupOne, false, FormMixed> {
    static constexpr int threads = 128, min_blocks = 7;
};
template <class F> struct PairShape<GroupOne, true, F> {
    static constexpr int threads = 256, min_blocks = 5;
};
// The block shapes an autotuner may choose instead (TileConfig::pair_block):
// 128 threads at 8 blocks per SM (7 in the mixed form's dense launch) or 256
// at 4 (5 in a list launch, whose kernel holds 48 registers).
template <class F, bool kList, int kT> struct PairBlock;
template <class F, bool kList> struct PairBlock<F, kList, 128> {
    static constexpr int threads = 128, min_blocks = (!kList && F::kMixed) ? 7 : 8;
};
template <class F, bool kList> struct PairBlock<F, kList, 256> {
    static constexpr int threads = 256, min_blocks = kList ? 5 : 4;
};
constexpr int kMaxPerCell = 24;  // staged particles per cell at most

// Particles per cell the pair pass stages (a tile with more falls back to the
// unstaged sweep, without lists): 1.2 times the lattice count (cell area /
// particle area), at least 8 - of the scene, or of a batch's densest scene -
// so that 7 or 8 blocks share an SM (13 to 13.5 per cell at h = 1.2 dx: 16
// or 17, 25 to 27 KB a block; a 16-cell tile stages about 700 of its 864 to
// 918 entries).  A sparse scene swept alone stages kMaxPerCell.
inline double lattice_per_cell(const sphnj_params &p) {
    if (p.fluid_number_total <= 0 || !(p.particle_diameter > 0.0f)) return 0.0;
    const double dx = p.particle_diameter;
    return (double)p.interval[0] * p.interval[1] / (dx * dx);
}
inline int staged_per_cell(double lattice) {
    return std::min(kMaxPerCell, std::max(8, (int)std::ceil(1.2 * lattice)));
}
inline int pair_per_cell(const GroupOne &g, bool list) {
    return list ? kMaxPerCell : staged_per_cell(lattice_per_cell(g.s.p));
}
inline int pair_per_cell(const GroupMany &g, bool) {
    double most = 0.0;
    for (int k = 0; k < g.n; ++k) most = std::max(most, lattice_per_cell(g.h_scenes[k].p));
    return staged_per_cell(most);
}
constexpr int kBlock = 256;
constexpr int kFallbackBlocks = 304;  // 2 x 152 SMs, grid-stride

__device__ __forceinline__ float fdiv(float a, float b) { return __fdividef(a, b); }
// sqrt by the SFU (PTX sqrt.approx.ftz.f32), the square root sqrtf becomes
// in the reference's -use_fast_math build
__device__ __forceinline__ float sqrt_approx(float x) {
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
// Eigen's normalized() (x / sqrt(|x|^2), zero vector unchanged) as the
// reference's fast-math build evaluates it in the pair terms
__device__ __forceinline__ float2 nrm_fast(float2 a) {
    float z = sqn(a);
    if (z > 0.0f) {
        float s = sqrt_approx(z);
        return make_float2(fdiv(a.x, s), fdiv(a.y, s));
    }
    return a;
}
__device__ __forceinline__ float by_phase(const float (&a)[2], int ph) { return ph ? a[1] : a[0]; }

// ---- where fluid neighbours come from ----------------------------------------
// key(t): handle of the t-th entry of a fluid range; the other members read
// that neighbour's fields.  Global: through the CSR index list.  Tile: from
// the block's shared-memory copy.
// x(k, sh): position of entry k in the sweep's frame; sh is the frame shift
// of the neighbour cell the entry was listed in (mixed form).
template <class F> struct SrcGlobal {
    const DevState *d;
    __device__ __forceinline__ int2 range(int, int2 r) const { return r; }
    __device__ __forceinline__ int key(int t) const { return __ldg(&d->lst_f[t]); }
    // (the list bodies, which call x(k) without a shift, take their entries
    // from a tile only; with a global source they return before reading)
    __device__ __forceinline__ float2 x(int k, float2 sh = float2()) const { return F::f_nbr(*d, k, sh); }
    __device__ __forceinline__ float2 x_byte(unsigned off) const { return x((int)(off >> 3)); }
    __device__ __forceinline__ float2 u(int k) const { return __ldg(&d->f_vel[k]); }
    __device__ __forceinline__ float rho(int k) const { return __ldg(&d->f_rho[k]); }
    __device__ __forceinline__ float pr(int k) const { return __ldg(&d->f_p[k]); }
    __device__ __forceinline__ int phase(int k) const { return __ldg(&d->f_phase[k]); }
    __device__ __forceinline__ int fbt(int k) const { return __ldg(&d->f_fbt[k]); }
    __device__ __forceinline__ int pid(int k) const { return k; }
};

// The shifting passes' fluid neighbours read by CSR position from the
// list-order positions (f_xl, in the frame of the cell they are listed in).
template <class F> struct SrcListOrder {
    const DevState *d;
    __device__ __forceinline__ int2 range(int, int2 r) const { return r; }
    __device__ __forceinline__ int key(int t) const { return t; }
    __device__ __forceinline__ float2 x(int t, float2 sh = float2()) const { return F::f_nbr_l(*d, t, sh); }
    __device__ __forceinline__ float2 x_byte(unsigned off) const { return x((int)(off >> 3)); }
};

struct SrcTile {
    const float2 *pos, *vel, *rp;  // rp = {rho, p}
    const uint8_t *flags;          // phase | boundary type << 1
    const int *idx;                // particle index of each staged entry
    const int *base, *off;         // per column strip: first CSR position, first slot
    __device__ __forceinline__ int2 range(int strip, int2 r) const {
        return make_int2(off[strip] + r.x - base[strip], r.y);
    }
    __device__ __forceinline__ int key(int t) const { return t; }
    __device__ __forceinline__ float2 x(int k, float2 = float2()) const { return pos[k]; }
    // position of the entry at byte offset 8 k (a neighbour-list entry)
    __device__ __forceinline__ float2 x_byte(unsigned off) const {
        return *reinterpret_cast<const float2 *>(reinterpret_cast<const char *>(pos) + off);
    }
    __device__ __forceinline__ float2 u(int k) const { return vel[k]; }
    __device__ __forceinline__ float rho(int k) const { return rp[k].x; }
    __device__ __forceinline__ float pr(int k) const { return rp[k].y; }
    __device__ __forceinline__ int phase(int k) const { return flags[k] & 1; }
    __device__ __forceinline__ int fbt(int k) const { return flags[k] >> 1; }
    __device__ __forceinline__ int pid(int k) const { return idx[k]; }
};

struct FAcc {
    float velo_div, color;
    float2 du_dt, grad;
    float4 du_dx;  // m00 m10 m01 m11
    int near;
};

// 1 / x and 1 / sqrt(x) by the SFU (PTX rcp.approx.ftz.f32, rsqrt.approx.ftz.f32)
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Products and accumulations of the pair and shifting terms.  The mixed form
// writes them with round-to-nearest intrinsics - a += x y as one explicit
// FMA, products rounded one by one - so that every kernel that inlines them
// (one-scene and batched launches, which have different block shapes and
// register budgets) rounds them the same way; the plain form leaves
// contraction to the compiler, as the reference's build does.
template <class F> __device__ __forceinline__ float mul2(float x, float y) {
    if constexpr (F::kMixed) return __fmul_rn(x, y);
    else return x * y;
}
template <class F> __device__ __forceinline__ void mad_to(float &a, float x, float y) {
    if constexpr (F::kMixed) a = __fmaf_rn(x, y, a);
    else a += x * y;
}

// x_j - x_i: two subtractions, packed in the mixed form (same results)
template <class F> __device__ __forceinline__ float2 sep(float2 xj, float2 xi) {
    if constexpr (F::kMixed) return sub2x(xj, xi);
    else return sub2(xj, xi);
}

// Riemann pair term shared by fluid, solid and virtual neighbours
// (fluid.cu:48-58, 115-124, 167-177).  The plain form divides as the
// reference's fast-math build does, one approximate division per '/'.  The
// mixed form takes one SFU reciprocal of rho_i + rho_j for the five divisions
// by it, reciprocals of rho_i and c_s (loop-invariant), and the direction
// from an SFU reciprocal square root: the same expressions with fewer SFU
// operations.
template <class F>
__device__ __forceinline__ void riemann(float2 u_i, float2 u_j, float p_i, float p_j, float rho_i, float rho_j,
                                        float cs, float2 dx, float kc, FAcc &a) {
    const float rs = rho_i + rho_j;
    float ps, am, t;
    float2 n, vs;
    if constexpr (F::kMixed) {
        const float irs = rcp_approx(rs);
        ps = __fmul_rn(sum2(rho_i, p_j, rho_j, p_i), irs);
        const float z = sqn(dx);
        const float iz = rsqrt_approx(z);
        n = z > 0.0f ? mul2x(dx, splat2(iz)) : dx;
        const float2 uij = sub2x(u_i, u_j);
        const float du = dot2(uij, n);
        if (du >= 0.0f)
            ps = __fadd_rn(ps, __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(rho_i, rho_j), du), irs),
                                         fminf(__fmul_rn(3.0f, du), cs)));
        // (rho_i u_i + rho_j u_j) / (rho_i + rho_j), per component
        // fma(rho_j, u_j, rho_i u_i) then times 1 / (rho_i + rho_j)
        vs = mul2x(fma2x(splat2(rho_j), u_j, mul2x(splat2(rho_i), u_i)), splat2(irs));
        t = __fmul_rn(__fmul_rn(__fsub_rn(p_i, p_j), irs), rcp_approx(cs));
        vs = fma2x(splat2(t), n, vs);
        am = __fmul_rn(ps, __fmul_rn(-2.0f, rcp_approx(rho_i)));  // = (-2 ps) / rho_i, one rounding
        // the sums, each product rounded and then one fused add, as mad_to:
        // in pairs of components (packed FP32)
        a.du_dt = fma2x(mul2x(splat2(am), dx), splat2(kc), a.du_dt);
        a.velo_div = __fmaf_rn(__fmul_rn(__fmul_rn(2.0f, rho_i), dot2(sub2x(u_i, vs), dx)), kc, a.velo_div);
        // (u_j - u_i) dx kc as (u_i - u_j) dx (-kc): the same value (a zero
        // difference may give the other zero sign)
        const float2 c0 = fma2x(mul2x(uij, splat2(dx.x)), splat2(-kc), make_float2(a.du_dx.x, a.du_dx.y));
        const float2 c1 = fma2x(mul2x(uij, splat2(dx.y)), splat2(-kc), make_float2(a.du_dx.z, a.du_dx.w));
        a.du_dx = make_float4(c0.x, c0.y, c1.x, c1.y);
        return;
    } else {
        ps = fdiv(sum2(rho_i, p_j, rho_j, p_i), rs);
        n = nrm_fast(dx);
        const float du = dot2(sub2(u_i, u_j), n);
        if (du >= 0.0f) ps += fdiv(rho_i * rho_j * du, rs) * fminf(3.0f * du, cs);
        vs = make_float2(fdiv(sum2(rho_i, u_i.x, rho_j, u_j.x), rs), fdiv(sum2(rho_i, u_i.y, rho_j, u_j.y), rs));
        t = fdiv(fdiv(p_i - p_j, rs), cs);
        vs.x += t * n.x;
        vs.y += t * n.y;
        am = fdiv(-2.0f * ps, rho_i);
    }
    mad_to<F>(a.du_dt.x, mul2<F>(am, dx.x), kc);
    mad_to<F>(a.du_dt.y, mul2<F>(am, dx.y), kc);
    mad_to<F>(a.velo_div, mul2<F>(mul2<F>(2.0f, rho_i), dot2(sub2(u_i, vs), dx)), kc);
    float2 w = sub2(u_j, u_i);
    mad_to<F>(a.du_dx.x, mul2<F>(w.x, dx.x), kc);
    mad_to<F>(a.du_dx.y, mul2<F>(w.y, dx.x), kc);
    mad_to<F>(a.du_dx.z, mul2<F>(w.x, dx.y), kc);
    mad_to<F>(a.du_dx.w, mul2<F>(w.y, dx.y), kc);
}

template <class F>
__device__ __forceinline__ void viscous(const sphnj_params &p, float2 u_i, float2 u_j, float rho_i, int ph_i,
                                        float2 dx, float kc, FAcc &a) {
    float vis = dot2(sub2(u_j, u_i), dx);
    float am;
    if constexpr (F::kMixed) {
        vis = __fmul_rn(vis, rcp_approx(__fmaf_rn(0.01f, p.smoothing_length_square, sqn(dx))));
        am = __fmul_rn(__fmul_rn(__fmul_rn(8.0f, by_phase(p.viscosity, ph_i)), vis), rcp_approx(rho_i));
    } else {
        vis = fdiv(vis, sqn(dx) + 0.01f * p.smoothing_length_square);
        am = fdiv(8.0f * by_phase(p.viscosity, ph_i) * vis, rho_i);
    }
    mad_to<F>(a.du_dt.x, mul2<F>(am, dx.x), kc);
    mad_to<F>(a.du_dt.y, mul2<F>(am, dx.y), kc);
}

// State of particle i that every pair term reads.
struct PairI {
    int i, ph;
    float2 x, u;
    float p, rho, cs;
};

__device__ __forceinline__ PairI load_pair_i(const sphnj_params &p, const DevState &d, int i, float2 x) {
    PairI s;
    s.i = i;
    s.x = x;
    s.u = d.f_vel[i];
    s.p = d.f_p[i];
    s.rho = d.f_rho[i];
    s.ph = d.f_phase[i];
    s.cs = by_phase(p.sound_speed, s.ph);
    return s;
}

__device__ __forceinline__ void zero(FAcc &a) {
    a.velo_div = 0.f;
    a.color = 0.f;
    a.du_dt = make_float2(0.f, 0.f);
    a.grad = make_float2(0.f, 0.f);
    a.du_dx = make_float4(0.f, 0.f, 0.f, 0.f);
    a.near = SPHNJ_NO_PARTICLE;
}

// fluidFluidCalculate (fluid.cu:25-80) for a neighbour inside the cutoff
template <class F, class Src>
__device__ __forceinline__ void fluid_term(const sphnj_params &p, const Src &src, int k, const PairI &s, float2 dx,
                                           FAcc &a) {
    const float R2 = p.impact_distance_square;
    const float kc = F::gw(p, sqn(dx));
    const float2 u_j = src.u(k);
    riemann<F>(s.u, u_j, s.p, src.pr(k), s.rho, src.rho(k), s.cs, dx, kc, a);
    const int ph_j = src.phase(k);
    if (!(s.ph == SPHNJ_LIQUID && ph_j == SPHNJ_GAS)) {
        mad_to<F>(a.color, dot2(dx, dx), kc);
        if constexpr (F::kMixed) {
            a.grad = fma2x(dx, splat2(kc), a.grad);
        } else {
            mad_to<F>(a.grad.x, dx.x, kc);
            mad_to<F>(a.grad.y, dx.y, kc);
        }
    }
    if (src.fbt(k) == SPHNJ_FREE_SURFACE && s.ph == SPHNJ_LIQUID && s.i != src.pid(k)) {
        if (sqn(dx) < 0.25f * R2) a.near = SPHNJ_HAS_NEAR_PARTICLE;
        else if (a.near == SPHNJ_NO_PARTICLE) a.near = SPHNJ_HAS_PARTICLE;
    }
    if (p.is_fluid_viscid) viscous<F>(p, s.u, u_j, s.rho, s.ph, dx, kc, a);
}

__device__ __forceinline__ void store_pair(const DevState &d, int i, const FAcc &a) {
    d.f_drho[i] = a.velo_div;
    d.f_dudt[i] = a.du_dt;
    d.f_near[i] = (uint8_t)a.near;
    d.f_color[i] = a.color;
    d.f_grad[i] = a.grad;
    d.f_dudx[i] = a.du_dx;
}

// ---- tile geometry ---------------------------------------------------------
// Block b owns home cells (ci, cj0 .. cj1-1) of one column.  Its fluid
// neighbours are the cells (ci-1..ci+1, cj0-1..cj1): per column one
// contiguous CSR range ("strip"), and so are its virtual neighbours.  The
// staged entries of a tile are its fluid strips at slots 0 .. total-1 and,
// in the shifting passes, its virtual strips after them (slots total ..
// total + total_v - 1) when both fit (virt_staged).
struct TileGeom {
    int home_b, home_e, total, total_v;
    int col, row0;  // the tile's column and first row (its frame origin in the mixed form)
};

// Per column strip s: first CSR position and first slot, of the fluid
// (base, off) and of the virtual entries (vbase, voff); in shared memory.
struct TileStrips {
    int base[3], off[3], vbase[3], voff[3];
};

// Whether a tile's virtual strips are staged (after its fluid strips) in a
// staging area of cap entries.  The pair pass stores virtual slots in the
// neighbour lists of the tile's particles exactly when the shifting passes,
// which see the same cell lists and the same cap, stage them.
__device__ __forceinline__ bool virt_staged(const TileGeom &g, int cap) { return g.total + g.total_v <= cap; }

__device__ __forceinline__ float list_radius2(const sphnj_params &p) {
    return p.impact_distance_square * ((1.0f + kSkin) * (1.0f + kSkin));
}

// Writes one particle's list: 16-bit entries (byte offset 8 t of tile slot
// t < 8192), in chunks of eight at col[c nf], through an 8-entry FIFO in four
// registers - each push shifts the 128-bit value down by 16 bits and inserts
// at the top, so after 8 pushes the first entry is in the low half of b0 and
// the full chunk goes out as one 16-byte store.
struct ListWriter {
    uint4 *col;
    size_t nf;
    unsigned b0 = 0u, b1 = 0u, b2 = 0u, b3 = 0u;
    int n = 0;
    __device__ __forceinline__ ListWriter(uint4 *c, size_t stride) : col(c), nf(stride) {}
    __device__ __forceinline__ void push(int t) {
        if (n < kNbrCap) {
            b0 = __funnelshift_r(b0, b1, 16);
            b1 = __funnelshift_r(b1, b2, 16);
            b2 = __funnelshift_r(b2, b3, 16);
            b3 = __funnelshift_r(b3, (unsigned)t << 3, 16);
            if ((n & 7) == 7) col[(n >> 3) * nf] = make_uint4(b0, b1, b2, b3);
        }
        ++n;
    }
    // stores the last, partial chunk; false when the list is over kNbrCap
    __device__ __forceinline__ bool finish() {
        if (n > kNbrCap) return false;
        if (n & 7) {  // move the partial chunk's entries to the low end
            for (int e = n & 7; e < 8; ++e) {
                b0 = __funnelshift_r(b0, b1, 16);
                b1 = __funnelshift_r(b1, b2, 16);
                b2 = __funnelshift_r(b2, b3, 16);
                b3 = b3 >> 16;
            }
            col[(n >> 3) * nf] = make_uint4(b0, b1, b2, b3);
        }
        return true;
    }
};

// findFluidPair for particle i (fluid.cu:193-254), in frame fr.  kRecord
// (tile source only): when vs is set, also writes the particle's list for
// the shifting passes through lw - every fluid and virtual candidate within
// the list radius, in the walk's order, the fluid ones by tile slot, the
// virtual ones by their slot in the tile's staged virtual strips vs.
template <class F, bool kRecord = false, class Src>
__device__ __forceinline__ void pair_particle(const sphnj_params &p, const DevState &d, const Src &src, int i,
                                              Frame fr, ListWriter *lw = nullptr, const TileStrips *vs = nullptr) {
    const int nf = p.fluid_number_total;
    const int nx = p.cell_number[0], ny = p.cell_number[1];
    const float R2 = p.impact_distance_square;
    [[maybe_unused]] const float Rs2 = list_radius2(p);
    const bool viscid = p.is_fluid_viscid != 0;
    const PairI si = load_pair_i(p, d, i, F::f_home(p, d, fr, i));
    const float2 x_i = si.x, u_i = si.u;
    const float p_i = si.p, rho_i = si.rho, cs = si.cs;
    const int ph_i = si.ph;
    const int c = d.f_cell[i];
    FAcc a;
    zero(a);
    for (int n = 0; n < 9; ++n) {
        const int m = neighbour_cell(c, n, nx, ny);
        if (m < 0) continue;
        const float2 sh = F::shift(p, fr, n);
        const int2 rf = src.range(n / 3, __ldg(&d.rng_f[m]));
        for (int t = rf.x; t < rf.x + rf.y; ++t) {
            const int k = src.key(t);
            const float2 dx = sub2(src.x(k, sh), x_i);
            if constexpr (kRecord)
                if (vs && sqn(dx) < Rs2) lw->push(k);  // a tile source's key is the slot
            if (sqn(dx) < R2) fluid_term<F>(p, src, k, si, dx, a);
        }
        const int2 rs = __ldg(&d.rng_s[m]);
        for (int t = rs.x; t < rs.x + rs.y; ++t) {
            const int j = __ldg(&d.lst_s[t]);
            const float2 dx = sub2(F::s_nbr(d, j, sh), x_i);
            if (!(sqn(dx) < R2)) continue;
            const float kc = F::gw(p, sqn(dx));
            const float2 u_j = F::s_vel(d, j);
            riemann<F>(u_i, u_j, p_i, __ldg(&d.s_p[j]), rho_i, rho_i, cs, dx, kc, a);
            mad_to<F>(a.grad.x, dx.x, kc);
            mad_to<F>(a.grad.y, dx.y, kc);
            if (viscid) viscous<F>(p, u_i, u_j, rho_i, ph_i, dx, kc, a);
        }
        const int2 rv = __ldg(&d.rng_v[m]);
        for (int t = rv.x; t < rv.x + rv.y; ++t) {
            const int j = __ldg(&d.lst_v[t]);
            const float2 dx = sub2(F::v_nbr(d, j, sh), x_i);
            if constexpr (kRecord)
                if (vs && sqn(dx) < Rs2) lw->push(vs->voff[n / 3] + t - vs->vbase[n / 3]);
            if (!(sqn(dx) < R2)) continue;
            const float kc = F::gw(p, sqn(dx));
            const float rho_j = by_phase(p.reference_density, __ldg(&d.v_phase[j]));
            const float2 u_j = __ldg(&d.v_vel[j]);
            riemann<F>(u_i, u_j, p_i, __ldg(&d.v_p[j]), rho_i, rho_j, cs, dx, kc, a);
            // fluid.cu:179 reads the fluid phase array with the virtual
            // index; past the fluid count it is taken as LIQUID.
            const int ph_j = j < nf ? (int)__ldg(&d.f_phase[j]) : SPHNJ_LIQUID;
            if (!(ph_i == SPHNJ_LIQUID && ph_j == SPHNJ_GAS)) {
                mad_to<F>(a.color, dot2(dx, dx), kc);
                mad_to<F>(a.grad.x, dx.x, kc);
                mad_to<F>(a.grad.y, dx.y, kc);
            }
            if (viscid) viscous<F>(p, u_i, u_j, rho_i, ph_i, dx, kc, a);
        }
    }
    store_pair(d, i, a);
}

// correctionCalculate for particle i (fluid.cu:316-367): its shifting gradient
// at x_i (in frame fr) in cell c
template <class F, class Src>
__device__ __forceinline__ float2 shift_particle(const sphnj_params &p, const DevState &d, const Src &src, float2 x_i,
                                                 int c, Frame fr) {
    const int nx = p.cell_number[0], ny = p.cell_number[1];
    const float R2 = p.impact_distance_square;
    float2 g = make_float2(0.f, 0.f);
    for (int n = 0; n < 9; ++n) {
        const int m = neighbour_cell(c, n, nx, ny);
        if (m < 0) continue;
        const float2 sh = F::shift(p, fr, n);
        const int2 rf = src.range(n / 3, __ldg(&d.rng_f[m]));
        for (int t = rf.x; t < rf.x + rf.y; ++t) {
            const float2 dx = sub2(src.x(src.key(t), sh), x_i);
            if (sqn(dx) < R2) {
                const float kc = F::gw_shift(p, sqn(dx));
                mad_to<F>(g.x, dx.x, kc);
                mad_to<F>(g.y, dx.y, kc);
            }
        }
        const int2 rs = __ldg(&d.rng_s[m]);
        for (int t = rs.x; t < rs.x + rs.y; ++t) {
            const float2 dx = sub2(F::s_nbr(d, __ldg(&d.lst_s[t]), sh), x_i);
            if (sqn(dx) < R2) {
                const float kc = F::gw_shift(p, sqn(dx));
                mad_to<F>(g.x, dx.x, kc);
                mad_to<F>(g.y, dx.y, kc);
            }
        }
        const int2 rv = __ldg(&d.rng_v[m]);
        for (int t = rv.x; t < rv.x + rv.y; ++t) {
            const float2 dx = sub2(F::v_nbr(d, __ldg(&d.lst_v[t]), sh), x_i);
            if (sqn(dx) < R2) {
                const float kc = F::gw_shift(p, sqn(dx));
                mad_to<F>(g.x, dx.x, kc);
                mad_to<F>(g.y, dx.y, kc);
            }
        }
    }
    if constexpr (F::kShiftScaled) g = make_float2(g.x * F::shift_scale(p), g.y * F::shift_scale(p));
    return g;
}

// ---- neighbour lists ----------------------------------------------------------
// When the 3x3 stencil of cell c holds only fluid entries, the stencil's
// candidates in the reference's order (slots 0..8, fluid/solid/virtual per
// cell) are exactly three contiguous CSR ranges, one per column (rows
// cj-1..cj+1 of a column are consecutive cell ids).  The pair pass records
// the tile slots of the candidates within cutoff * (1 + kSkin), in that
// order; the pair terms and the shifting passes of the same step visit only
// those entries - in the same order, with the exact cutoff test - while the
// positions have moved by less than half the skin.  The tile staging is the
// same in every pass of a step (same lists, same tile height), so the slots
// stay valid.  A particle next to a wall (virtual entries in its stencil,
// no solid ones) gets a list for the shifting passes too, cell by cell -
// the fluid entries of a cell, then its virtual entries, as the stencil
// walk visits them - with virtual slots in the staging of its tile.
struct Strips {
    int base[3], len[3];
};

// What a particle's stencil holds (strips_of): only fluid entries; fluid
// and virtual entries; or something that takes the stencil walk (solid
// entries, or a column strip of more than 64 fluid entries).
enum StencilKind { kStencilFluid = 0, kStencilVirt = 1, kStencilWalk = 2 };

__device__ __forceinline__ Strips strips_of(const sphnj_params &p, const DevState &d, int c, int &kind) {
    const int nx = p.cell_number[0], ny = p.cell_number[1];
    const int ci = c / ny, cj = c - ci * ny;
    const int r0 = max(cj - 1, 0), r1 = min(cj + 1, ny - 1);
    Strips S;
    bool walk = false, virt = false;
#pragma unroll
    for (int s = 0; s < 3; ++s) {
        const int col = ci + s - 1;
        S.base[s] = 0;
        S.len[s] = 0;
        if (col < 0 || col >= nx) continue;
        const int2 a = __ldg(&d.rng_f[col * ny + r0]), b = __ldg(&d.rng_f[col * ny + r1]);
        S.base[s] = a.x;
        S.len[s] = b.x + b.y - a.x;
        if (S.len[s] > 64) walk = true;
        for (int r = r0; r <= r1; ++r) {
            const int m = col * ny + r;
            if (__ldg(&d.rng_s[m]).y) walk = true;
            if (__ldg(&d.rng_v[m]).y) virt = true;
        }
    }
    kind = walk ? kStencilWalk : virt ? kStencilVirt : kStencilFluid;
    return S;
}

// Pair pass for particle i at CSR position h; records its neighbour list
// when `listable` (its tile was staged, so the source is the tile).  vs:
// the tile's virtual strips when the shifting passes stage them (else null).
template <class F, class Src>
__device__ __forceinline__ void pair_particle_listed(const sphnj_params &p, const DevState &d, const Src &src, int i,
                                                     int h, bool listable, Frame fr, const TileStrips *vs) {
    int kind = kStencilWalk;
    Strips S;
    if (listable) S = strips_of(p, d, d.f_cell[i], kind);
    if (kind != kStencilFluid) {
        // the pair terms by the stencil walk, which next to a wall also
        // records the list of the shifting passes
        if constexpr (std::is_same<Src, SrcTile>::value) {
            const TileStrips *rec = kind == kStencilVirt ? vs : nullptr;
            ListWriter lw(d.f_nbr + h, (size_t)p.fluid_number_total);
            pair_particle<F, true>(p, d, src, i, fr, &lw, rec);
            d.f_nbr_cnt[h] = rec && lw.finish() ? (uint8_t)lw.n : kNbrNone;
        } else {
            d.f_nbr_cnt[h] = kNbrNone;
            pair_particle<F>(p, d, src, i, fr);
        }
        return;
    }
    const float R2 = p.impact_distance_square, Rs2 = list_radius2(p);
    const PairI si = load_pair_i(p, d, i, F::f_home(p, d, fr, i));
    const size_t nf = (size_t)p.fluid_number_total;
    uint4 *col = d.f_nbr + h;  // chunk c at col[c nf]
    ListWriter lw(col, nf);
#pragma unroll
    for (int s = 0; s < 3; ++s) {
        const int2 rr = src.range(s, make_int2(S.base[s], S.len[s]));
        for (int t = rr.x; t < rr.x + rr.y; ++t)
            if (sqn(sep<F>(src.x(src.key(t)), si.x)) < Rs2) lw.push(t);
    }
    if (!lw.finish()) {
        d.f_nbr_cnt[h] = kNbrNone;
        pair_particle<F>(p, d, src, i, fr);
        return;
    }
    const int n = lw.n;
    d.f_nbr_cnt[h] = (uint8_t)n;
    FAcc a;
    zero(a);
    for (int c = 0; c < n; c += 8) {
        const uint4 v = col[(c >> 3) * nf];
        const unsigned w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            if (c + e < n) {
                const int k = src.key((int)(((w[e >> 1] >> (16 * (e & 1))) & 0xFFFFu) >> 3));
                const float2 dx = sep<F>(src.x(k), si.x);
                if (sqn(dx) < R2) fluid_term<F>(p, src, k, si, dx, a);
            }
        }
    }
    store_pair(d, i, a);
}

// Shifting gradient of the particle at CSR position h, at x_i in cell c,
// through its neighbour list when use_list (and it has one).
template <class F, class Src>
__device__ __forceinline__ float2 shift_particle_listed(const sphnj_params &p, const DevState &d, const Src &src,
                                                        int h, bool use_list, float2 x_i, int c, Frame fr) {
    const size_t nf = (size_t)p.fluid_number_total;
    const uint4 *col = d.f_nbr + h;  // chunk c at col[c nf]
    // the first chunk is loaded together with the count (the list array
    // always holds it), so that the two loads share one memory latency
    const uint4 first = __ldg(col);
    const int n = use_list ? (int)d.f_nbr_cnt[h] : (int)kNbrNone;
    if (n == kNbrNone) return shift_particle<F>(p, d, src, x_i, c, fr);
    const float R2 = p.impact_distance_square;
    float2 g = make_float2(0.f, 0.f);
    // entries e < m of one chunk, in order (m = 8 for the full chunks, which
    // need no per-entry count test)
    auto chunk = [&](uint4 v, int m) {
        const unsigned w[4] = {v.x, v.y, v.z, v.w};
        float2 x_j[8];
#pragma unroll
        for (int e = 0; e < 8; ++e)  // all eight loads in flight first
            x_j[e] = src.x_byte((w[e >> 1] >> (16 * (e & 1))) & 0xFFFFu);
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            if (e < m) {
                const float2 dx = sep<F>(x_j[e], x_i);
                if (sqn(dx) < R2) {
                    const float kc = F::gw_shift(p, sqn(dx));
                    if constexpr (F::kMixed) {
                        g = fma2x(dx, splat2(kc), g);
                    } else {
                        mad_to<F>(g.x, dx.x, kc);
                        mad_to<F>(g.y, dx.y, kc);
                    }
                }
            }
        }
    };
    // the other chunks are prefetched into L1 as soon as the count is known
    // (4.15M dam break: shifting stage 2.079 -> 1.989 ms/step with the first
    // chunk's early load), and each chunk's load is issued one chunk ahead
    // of its use
    const int full = n >> 3;
    for (int k = 1; 8 * k < n; ++k) asm volatile("prefetch.global.L1 [%0];" ::"l"(col + k * nf));
    uint4 next = first;
    for (int c = 0; c < full; ++c) {
        const uint4 v = next;
        if (8 * (c + 1) < n) next = __ldg(col + (c + 1) * nf);
        chunk(v, 8);
    }
    if (n & 7) chunk(next, n & 7);
    if constexpr (F::kShiftScaled) g = make_float2(g.x * F::shift_scale(p), g.y * F::shift_scale(p));
    return g;
}

// The lists of this step still hold every pair within the cutoff when twice
// the summed per-update maximum displacement since the pair pass is inside
// the skin (margin 0.9 for rounding).  `pass` shifting updates came before.
// Lane k loads the maximum of update k, so the maxima arrive together rather
// than one after another; the butterfly sum leaves the same bits in every
// lane (each step adds the same two values).  Called by full warps.
__device__ __forceinline__ bool lists_valid(const sphnj_params &p, const DevState &d, int pass) {
    static_assert(kMaskShifts <= 32, "one lane per tracked update");
    if (pass >= kMaskShifts) return false;
    const int lane = threadIdx.x & 31;
    float moved = lane <= pass ? sqrtf(__uint_as_float(__ldcg(&d.disp2_bits[lane]))) : 0.0f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) moved += __shfl_xor_sync(0xffffffffu, moved, o);
    return 2.0f * moved < 0.9f * kSkin * sqrtf(p.impact_distance_square);
}
// The same test in two halves, for a kernel that issues the loads on entry
// (list_moved_share) and sums only when it first needs the answer.
__device__ __forceinline__ unsigned int list_moved_share(const DevState &d, int pass) {
    const int lane = threadIdx.x & 31;
    return pass < kMaskShifts && lane <= pass ? __ldcg(&d.disp2_bits[lane]) : 0u;
}
__device__ __forceinline__ bool lists_valid(const sphnj_params &p, unsigned int share, int pass) {
    if (pass >= kMaskShifts) return false;
    float moved = sqrtf(__uint_as_float(share));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) moved += __shfl_xor_sync(0xffffffffu, moved, o);
    return 2.0f * moved < 0.9f * kSkin * sqrtf(p.impact_distance_square);
}

// Block-wide max of non-negative float bits, one atomicMax per block.
template <int kThreads>
__device__ __forceinline__ void block_max_to(unsigned int v, unsigned int *dst) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    __shared__ unsigned int wmax[kThreads / 32];
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        unsigned int w = threadIdx.x < kThreads / 32 ? wmax[threadIdx.x] : 0u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) w = max(w, __shfl_xor_sync(0xffffffffu, w, o));
        if (threadIdx.x == 0 && w) atomicMax(dst, w);
    }
}

// Warp-wide max of non-negative float bits with no block barrier (so a warp
// that finishes its particles early does not wait for the block's slowest):
// lane 0 issues the atomicMax only when the value already in *dst is smaller.
// *dst only grows while the max is taken, so a stale read costs at most a
// redundant atomic.  All 32 lanes of the warp call it.
__device__ __forceinline__ void warp_max_to(unsigned int v, unsigned int *dst) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0 && v > __ldcg(dst)) atomicMax(dst, v);
}

__device__ __forceinline__ unsigned int disp2(float2 a, float2 b) {
    const float dx = b.x - a.x, dy = b.y - a.y;
    const float v = dx * dx + dy * dy;
    return v == v ? __float_as_uint(v) : 0x7f800000u;  // NaN: treat as unbounded
}

// (I - n n^T) d with n = normalize(g), zeroed below EPS_FOR_SUM
// (fluid.cu:394-397)
// (the mixed form with round-to-nearest intrinsics, as mad_to)
template <class F> __device__ __forceinline__ float2 project(float2 g, float2 disp) {
    float2 n = normalized(g);
    if (sqrtf(sqn(n)) < EPS_FOR_SUM) n = make_float2(0.f, 0.f);
    if constexpr (F::kMixed) {
        const float m00 = __fsub_rn(1.0f, __fmul_rn(n.x, n.x)), m10 = -__fmul_rn(n.y, n.x),
                    m01 = -__fmul_rn(n.x, n.y), m11 = __fsub_rn(1.0f, __fmul_rn(n.y, n.y));
        return make_float2(sum2(m00, disp.x, m01, disp.y), sum2(m10, disp.x, m11, disp.y));
    } else {
        float m00 = 1.0f - n.x * n.x, m10 = 0.0f - n.y * n.x, m01 = 0.0f - n.x * n.y, m11 = 1.0f - n.y * n.y;
        return make_float2(m00 * disp.x + m01 * disp.y, m10 * disp.x + m11 * disp.y);
    }
}

// Boundary type of a fluid particle as the shifting update assigns it
// (shiftDisplacementCalculate, fluid.cu:380-412): a function of its phase,
// colour and near flag, which only the pair pass sets, so it is the same in
// every pass of a step (the listed particles' types are computed once, in
// list order, before the first pass).
__device__ __forceinline__ uint8_t shift_class(int ph, float color, int near) {
    if (ph == SPHNJ_GAS) return SPHNJ_INNER;
    if (color < 1.5f) return near == SPHNJ_NO_PARTICLE ? SPHNJ_SPLASH : SPHNJ_FREE_SURFACE;
    if (color < 2.0f && near == SPHNJ_HAS_NEAR_PARTICLE) return SPHNJ_VICINITY;
    return SPHNJ_INNER;
}

// shiftDisplacementCalculate + correctionUpdate (fluid.cu:369-427) for one
// particle with shifting gradient g, done by the thread that computed g.
// A listed particle is addressed by its CSR position k (i < 0: its index is
// read from the list only where a particle-order field is touched); an
// unlisted one by its index, k = i.  The pass reads the position from xin[k]
// and writes the shifted one to xout[k] - the list-order pair f_xl / f_xl_alt
// for a listed particle, f_pos (f_off in the mixed form) / f_x_alt otherwise -
// so that every other particle's gradient in this pass still sees the
// positions before the update; the boundary type, the velocity, the
// compensations and the gradient are only ever read by the particle's own
// thread during the shifting passes and are updated in place.  Returns the
// squared displacement (float bits).
template <class F>
__device__ __forceinline__ unsigned int shift_update_particle(const sphnj_params &p, const DevState &d, int i, int k,
                                                              float2 g, const float2 *xin, float2 *xout, bool last,
                                                              bool listed) {
    auto index = [&] { return i >= 0 ? i : __ldg(&d.lst_f[k]); };
    // getMaxSpeed's clamp, fluid.cu:438-439
    const float vmax = __fsqrt_rn(__uint_as_float(*d.max_speed2_bits));
    const float max_speed = fminf(vmax, __fmul_rn(0.1f, fminf(p.sound_speed[0], p.sound_speed[1])));
    const float s = -p.particle_shift_coef * p.smoothing_length * p.dt;
    const float2 disp = make_float2(s * g.x, s * g.y);
    const uint8_t bt = listed ? d.f_btl[k] : shift_class(d.f_phase[i], d.f_color[i], d.f_near[i]);
    float2 dd;
    if (bt == SPHNJ_SPLASH) dd = make_float2(0.f, 0.f);
    else if (bt == SPHNJ_FREE_SURFACE || bt == SPHNJ_VICINITY) dd = project<F>(g, disp);
    else dd = disp;
    // the gradient and boundary type are state only after the step's last
    // pass (no pass reads them): earlier passes skip the two stores
    // (4.15M dam break: shifting stage 1.985 -> 1.953 ms/step)
    if (last) {
        const int ii = index();
        d.f_grad[ii] = g;
        d.f_fbt[ii] = bt;
    }
    const float2 sh = make_float2(max_speed * dd.x, max_speed * dd.y);
    if constexpr (F::kMixed) {
        float2 *const cp = listed ? d.f_offcl + k : d.f_offc + i;
        float2 x = xin[k], xc = *cp;
        const float2 x0 = x;
        kahan_add2(x, xc, sh);
        xout[k] = x;
        *cp = xc;
        // the velocity correction is linear in the shift with the pair
        // pass's du_dx, which no pass changes: a listed particle takes the
        // sum of its passes' corrections once, in the last pass, from its
        // total displacement (offset and compensation differences against
        // the values gathered before the first pass; the cell is the same in
        // every pass); an unlisted particle takes one per pass
        if (!listed || last) {
            float2 dx = sh;
            if (listed) {
                const float2 s0 = d.f_x0l[k], c0 = d.f_xc0l[k];
                dx = make_float2(__fsub_rn(__fsub_rn(x.x, s0.x), __fsub_rn(xc.x, c0.x)),
                                 __fsub_rn(__fsub_rn(x.y, s0.y), __fsub_rn(xc.y, c0.y)));
            }
            const int ii = index();
            const float4 m = d.f_dudx[ii];
            float2 v = d.f_vel[ii], vc = d.f_velc[ii];
            kahan_add2(v, vc, make_float2(sum2(m.x, dx.x, m.z, dx.y), sum2(m.y, dx.x, m.w, dx.y)));
            d.f_vel[ii] = v;
            d.f_velc[ii] = vc;
        }
        return disp2(x0, x);
    } else {
        const int ii = index();
        const float4 m = d.f_dudx[ii];
        const float2 x0 = xin[k];
        float2 x = x0;
        x.x += sh.x;
        x.y += sh.y;
        xout[k] = x;
        float2 v = d.f_vel[ii];
        v.x += m.x * sh.x + m.z * sh.y;
        v.y += m.y * sh.x + m.w * sh.y;
        d.f_vel[ii] = v;
        return disp2(x0, x);
    }
}

// ---- tiles ---------------------------------------------------------------
__device__ __forceinline__ bool tile_setup(const sphnj_params &p, const DevState &d, int blk, int tile_h,
                                           TileStrips &ts, TileGeom &g) {
    const int nx = p.cell_number[0], ny = p.cell_number[1];
    const int tiles_y = (ny + tile_h - 1) / tile_h;
    const int ci = blk / tiles_y, cj0 = (blk - ci * tiles_y) * tile_h;
    const int cj1 = min(cj0 + tile_h, ny);
    g.col = ci;
    g.row0 = cj0;
    const int2 h0 = __ldg(&d.rng_f[ci * ny + cj0]), h1 = __ldg(&d.rng_f[ci * ny + cj1 - 1]);
    g.home_b = h0.x;
    g.home_e = h1.x + h1.y;
    if (g.home_e <= g.home_b) return false;
    __shared__ int s_len[6];
    if (threadIdx.x < 3) {
        const int col = ci + (int)threadIdx.x - 1;
        int base = 0, len = 0, vbase = 0, vlen = 0;
        if (col >= 0 && col < nx) {
            const int r0 = max(cj0 - 1, 0), r1 = min(cj1, ny - 1);
            const int2 a = __ldg(&d.rng_f[col * ny + r0]), b = __ldg(&d.rng_f[col * ny + r1]);
            const int2 va = __ldg(&d.rng_v[col * ny + r0]), vb = __ldg(&d.rng_v[col * ny + r1]);
            base = a.x;
            len = b.x + b.y - a.x;
            vbase = va.x;
            vlen = vb.x + vb.y - va.x;
        }
        ts.base[threadIdx.x] = base;
        ts.vbase[threadIdx.x] = vbase;
        s_len[threadIdx.x] = len;
        s_len[3 + threadIdx.x] = vlen;
    }
    __syncthreads();
    g.total = s_len[0] + s_len[1] + s_len[2];
    g.total_v = s_len[3] + s_len[4] + s_len[5];
    if (threadIdx.x == 0) {
        ts.off[0] = 0;
        ts.off[1] = s_len[0];
        ts.off[2] = s_len[0] + s_len[1];
        ts.voff[0] = g.total;
        ts.voff[1] = g.total + s_len[3];
        ts.voff[2] = g.total + s_len[3] + s_len[4];
    }
    __syncthreads();
    return true;
}

__device__ __forceinline__ int tile_strip(const int *s_off, int k) { return k < s_off[1] ? 0 : (k < s_off[2] ? 1 : 2); }

// Position of fluid particle j, listed in column strip s of tile g, as the
// tile stages it: absolute (plain) or relative to the tile's origin cell
// (mixed).
template <class F>
__device__ __forceinline__ float2 tile_pos(const sphnj_params &p, const DevState &d, const TileGeom &g, int s, int j) {
    if constexpr (F::kMixed) {
        const int col = g.col + s - 1;
        const int row = __ldg(&d.f_cell[j]) - col * p.cell_number[1];
        return add2_rn(__ldg(&d.f_off[j]), cells_to_len(p, s - 1, row - g.row0));
    } else {
        return __ldg(&d.f_pos[j]);
    }
}

// The same for the entry at CSR position t, from the shifting passes'
// list-order positions and cells (contiguous reads over a strip).
template <class F>
__device__ __forceinline__ float2 tile_pos_l(const sphnj_params &p, const DevState &d, const TileGeom &g, int s,
                                             int t) {
    if constexpr (F::kMixed) {
        const int col = g.col + s - 1;
        const int row = __ldg(&d.f_celll[t]) - col * p.cell_number[1];
        return add2_rn(__ldg(&d.f_xl[t]), cells_to_len(p, s - 1, row - g.row0));
    } else {
        return __ldg(&d.f_xl[t]);
    }
}

// The same for the virtual entry at CSR position t of column strip s: its
// position as the stencil walk of a home particle of the tile forms it
// (F::v_nbr with the frame shift of its cell, which is v_cell[j]: the
// virtual particles keep the cells they were listed by).
template <class F>
__device__ __forceinline__ float2 tile_vpos(const sphnj_params &p, const DevState &d, const TileGeom &g, int s,
                                            int t) {
    const int j = __ldg(&d.lst_v[t]);
    if constexpr (F::kMixed) {
        const int col = g.col + s - 1;
        const int row = __ldg(&d.v_cell[j]) - col * p.cell_number[1];
        return F::v_nbr(d, j, cells_to_len(p, s - 1, row - g.row0));
    } else {
        return F::v_nbr(d, j, make_float2(0.f, 0.f));
    }
}

// Frame of home particle i in tile g (mixed form: the tile's origin cell).
template <class F>
__device__ __forceinline__ Frame tile_frame(const sphnj_params &p, const DevState &d, const TileGeom &g, int i) {
    if constexpr (F::kMixed) return Frame{0, d.f_cell[i] - g.col * p.cell_number[1] - g.row0};
    else return Frame{0, 0};
}
// ... of the home particle with cell c (its list-order cell)
template <class F>
__device__ __forceinline__ Frame tile_frame_c(const sphnj_params &p, const TileGeom &g, int c) {
    if constexpr (F::kMixed) return Frame{0, c - g.col * p.cell_number[1] - g.row0};
    else return Frame{0, 0};
}

// kList: the blocks loop over the scene's listed active tiles (batched
// launches, and scenes that sweep_compacted() selects); otherwise block b
// sweeps tile b, returning at once if it is empty.
template <class G, class F, bool kList, int kThreads, int kMinBlocks>
__global__ void __launch_bounds__(kThreads, kMinBlocks)
    k_fluid_pair_tiled(const __grid_constant__ G gs, int cap, int shift_cap) {
    int n_active = 0;
    SPHNJ_SCENE_SWEEP(gs, kList, n_active);
    const int tile_h = S.tile_h, use_lists = S.lists;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ TileStrips ts;
    float2 *s_pos = reinterpret_cast<float2 *>(smem);
    float2 *s_vel = s_pos + cap;
    float2 *s_rp = s_vel + cap;
    int *s_idx = reinterpret_cast<int *>(s_rp + cap);
    uint8_t *s_fl = reinterpret_cast<uint8_t *>(s_idx + cap);
    auto sweep = [&](int tile) {
        TileGeom g;
        if (!tile_setup(p, d, tile, tile_h, ts, g)) return;
        const bool staged = g.total <= cap;
        if (staged) {
            for (int k = threadIdx.x; k < g.total; k += blockDim.x) {
                const int s = tile_strip(ts.off, k);
                const int j = __ldg(&d.lst_f[ts.base[s] + k - ts.off[s]]);
                s_pos[k] = tile_pos<F>(p, d, g, s, j);
                s_vel[k] = __ldg(&d.f_vel[j]);
                s_rp[k] = make_float2(__ldg(&d.f_rho[j]), __ldg(&d.f_p[j]));
                s_idx[k] = j;
                s_fl[k] = (uint8_t)(__ldg(&d.f_phase[j]) | (__ldg(&d.f_fbt[j]) << 1));
            }
        }
        __syncthreads();
        if (staged) {
            const SrcTile src{s_pos, s_vel, s_rp, s_fl, s_idx, ts.base, ts.off};
            // the shifting passes stage this tile's virtual strips too: its
            // particles next to a wall get lists with virtual slots
            const TileStrips *vs = virt_staged(g, shift_cap) ? &ts : nullptr;
            for (int h = g.home_b + threadIdx.x; h < g.home_e; h += blockDim.x) {
                const int i = d.lst_f[h];
                pair_particle_listed<F>(p, d, src, i, h, use_lists != 0, tile_frame<F>(p, d, g, i), vs);
            }
        } else {
            const SrcGlobal<F> src{&d};
            for (int h = g.home_b + threadIdx.x; h < g.home_e; h += blockDim.x)
                pair_particle_listed<F>(p, d, src, d.lst_f[h], h, false, Frame{0, 0}, nullptr);
        }
    };
    if constexpr (kList) {
        for (int a = blk; a < n_active; a += nblk) {
            sweep(__ldg(&d.tile_list[a]));
            __syncthreads();  // the next tile overwrites the staged entries
        }
    } else {
        sweep(blk);
    }
}

// One shifting pass over the listed particles: each home particle's gradient,
// then its position update (shift_update_particle) by the same thread.
// kThreads per block at full occupancy, 32 registers (a small spill): 32
// registers at 8 blocks of 256 measured 4% faster than 40 at 6.  Batched
// launches over the active-tile lists and dense scenes use blocks of 128
// threads (kListBlock, kDenseBlock): a smaller block leaves fewer warps
// waiting at the tile's barriers while the others work (256-scene mixed
// sweep: 4.81 -> 4.52 ms/step; 4.15M dam break: 3.92 -> 3.80).
template <class G, class F, bool kList, int kThreads>
__global__ void __launch_bounds__(kThreads, 2048 / kThreads)
    k_shift_gradient_tiled(const __grid_constant__ G gs, int cap, int pass) {
    int n_active = 0;
    SPHNJ_SCENE_SWEEP(gs, kList, n_active);
    const int tile_h = S.tile_h;
    const bool last = pass + 1 >= p.shift_per_step;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ TileStrips ts;
    float2 *s_pos = reinterpret_cast<float2 *>(smem);
    // A block of a list launch, which sweeps several tiles, sums on its first
    // tile with work, after that tile's setup has issued its loads; a block
    // of one tile sums on entry (measured: each the faster of the two for its
    // launch shape).
    const bool entry_ok = kList ? false : lists_valid(p, d, pass);
    [[maybe_unused]] const unsigned int moved_share = kList ? list_moved_share(d, pass) : 0u;
    int first_ok = -1;
    unsigned int moved2 = 0u;
    auto sweep = [&](int tile) {
        TileGeom g;
        if (!tile_setup(p, d, tile, tile_h, ts, g)) return;
        // every thread of the block is here (tile_setup returns uniformly)
        if constexpr (kList)
            if (first_ok < 0) first_ok = lists_valid(p, moved_share, pass) ? 1 : 0;
        const bool use_list = kList ? first_ok != 0 : entry_ok;
        const bool staged = g.total <= cap;
        if (staged) {
            // the fluid strips, then (when they fit) the virtual strips, which
            // the lists of the tile's particles next to a wall refer to
            const int n_staged = virt_staged(g, cap) ? g.total + g.total_v : g.total;
            for (int k = threadIdx.x; k < n_staged; k += blockDim.x) {
                if (k < g.total) {
                    const int s = tile_strip(ts.off, k);
                    s_pos[k] = tile_pos_l<F>(p, d, g, s, ts.base[s] + k - ts.off[s]);
                } else {
                    const int s = tile_strip(ts.voff, k);
                    s_pos[k] = tile_vpos<F>(p, d, g, s, ts.vbase[s] + k - ts.voff[s]);
                }
            }
        }
        __syncthreads();
        if (staged) {
            const SrcTile src{s_pos, nullptr, nullptr, nullptr, nullptr, ts.base, ts.off};
            for (int h = g.home_b + threadIdx.x; h < g.home_e; h += blockDim.x) {
                const int c = d.f_celll[h];
                const Frame fr = tile_frame_c<F>(p, g, c);
                const float2 gr =
                    shift_particle_listed<F>(p, d, src, h, use_list, F::f_home_l(p, d, fr, h), c, fr);
                moved2 = max(moved2, shift_update_particle<F>(p, d, -1, h, gr, d.f_xl, d.f_xl_alt, last, true));
            }
        } else {
            // a tile the pair pass could not stage has no lists either
            const SrcListOrder<F> src{&d};
            for (int h = g.home_b + threadIdx.x; h < g.home_e; h += blockDim.x) {
                const float2 gr = shift_particle_listed<F>(p, d, src, h, false, F::f_home_l(p, d, Frame{0, 0}, h),
                                                           d.f_celll[h], Frame{0, 0});
                moved2 = max(moved2, shift_update_particle<F>(p, d, -1, h, gr, d.f_xl, d.f_xl_alt, last, true));
            }
        }
    };
    if constexpr (kList) {
        for (int a = blk; a < n_active; a += nblk) {
            sweep(__ldg(&d.tile_list[a]));
            __syncthreads();  // the next tile overwrites the staged entries
        }
    } else {
        sweep(blk);
    }
    if (pass < kMaskShifts) warp_max_to(moved2, &d.disp2_bits[1 + pass]);
}

// Per-particle forms: every particle (listed == null), or only the particles
// that are in no cell list.
template <class G, class F>
__global__ void __launch_bounds__(kPairBlock) k_fluid_pair_each(const __grid_constant__ G g, int only_unlisted) {
    SPHNJ_SCENE(g);
    const int nf = p.fluid_number_total;
    if (only_unlisted && *d.f_listed_total == nf) return;
    const int stamp = *d.stamp;
    const SrcGlobal<F> src{&d};
    for (int i = blk * blockDim.x + threadIdx.x; i < nf; i += nblk * blockDim.x)
        if (!only_unlisted || d.f_listed[i] != stamp) pair_particle<F>(p, d, src, i, Frame{0, 0});
}

// The shifting pass one thread per particle: the listed particles by their
// CSR position, from the list-order positions (only_unlisted 0: the untiled
// sweep), or the particles in no list, by index, from the particle arrays
// (only_unlisted 1).  Fluid neighbours are read in list order either way.
template <class G, class F>
__global__ void __launch_bounds__(kPairBlock) k_shift_gradient_each(const __grid_constant__ G g, int only_unlisted,
                                                                   int pass) {
    SPHNJ_SCENE(g);
    const int nf = p.fluid_number_total;
    const int listed = *d.f_listed_total;
    if (only_unlisted && listed == nf) return;
    const bool last = pass + 1 >= p.shift_per_step;
    const SrcListOrder<F> src{&d};
    unsigned int moved2 = 0u;
    if (only_unlisted) {
        const int stamp = *d.stamp;
        float2 *const x = F::kMixed ? d.f_off : d.f_pos;
        for (int i = blk * blockDim.x + threadIdx.x; i < nf; i += nblk * blockDim.x)
            if (d.f_listed[i] != stamp) {
                const float2 gr = shift_particle<F>(p, d, src, F::f_home(p, d, Frame{0, 0}, i), d.f_cell[i],
                                                    Frame{0, 0});
                moved2 = max(moved2, shift_update_particle<F>(p, d, i, i, gr, x, d.f_x_alt, last, false));
            }
    } else {
        for (int h = blk * blockDim.x + threadIdx.x; h < listed; h += nblk * blockDim.x) {
            const float2 gr = shift_particle<F>(p, d, src, F::f_home_l(p, d, Frame{0, 0}, h), d.f_celll[h],
                                                Frame{0, 0});
            moved2 = max(moved2, shift_update_particle<F>(p, d, -1, h, gr, d.f_xl, d.f_xl_alt, last, true));
        }
    }
    if (pass < kMaskShifts) warp_max_to(moved2, &d.disp2_bits[1 + pass]);
}

// Before the first shifting pass: the listed particles' positions (f_pos,
// f_off in the mixed form), cells and boundary types into list order (in the
// mixed form also the offset compensations, and both offset and compensation
// once more as the start of the total displacement).
template <class G, class F> __global__ void __launch_bounds__(kBlock) k_shift_gather(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const int h = blk * blockDim.x + threadIdx.x;
    if (p.shift_per_step <= 0 || h >= *d.f_listed_total) return;
    const int i = __ldg(&d.lst_f[h]);
    const float2 x = (F::kMixed ? d.f_off : d.f_pos)[i];
    d.f_xl[h] = x;
    d.f_celll[h] = __ldg(&d.f_cell[i]);
    d.f_btl[h] = shift_class(d.f_phase[i], d.f_color[i], d.f_near[i]);
    if constexpr (F::kMixed) {
        const float2 xc = d.f_offc[i];
        d.f_offcl[h] = xc;
        d.f_x0l[h] = x;
        d.f_xc0l[h] = xc;
    }
}

// After the last one (and the copy back of the unlisted particles after an
// odd number of passes): the listed particles' positions (and offset
// compensations) back to the particle arrays, from the list-order buffers.
template <class G, class F> __global__ void __launch_bounds__(kBlock) k_shift_scatter(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const int h = blk * blockDim.x + threadIdx.x;
    if (p.shift_per_step <= 0 || h >= *d.f_listed_total) return;
    const float2 *x = (p.shift_per_step & 1) ? d.f_xl_alt : d.f_xl;
    const int i = __ldg(&d.lst_f[h]);
    (F::kMixed ? d.f_off : d.f_pos)[i] = x[h];
    if constexpr (F::kMixed) d.f_offc[i] = d.f_offcl[h];
}

// densityToPressure, fluid.cu:15-23
__device__ __forceinline__ float density_to_pressure(const sphnj_params &p, float rho, int ph) {
    float pr = (powf(rho * by_phase(p.reference_density_inverse, ph), by_phase(p.gamma, ph)) - 1.0f) *
               by_phase(p.coefficient_rho2p, ph);
    return fmaxf(pr, p.min_pressure);
}

// Lower-left corner of cell c, relative to the domain box: the box bounds in
// the frame of cell c (mixed form), for the position clamp.
__device__ __forceinline__ float4 box_in_cell(const sphnj_params &p, int c) {
    const int ny = p.cell_number[1];
    const int cx = c / ny, cy = c - cx * ny;
    const float ox = __fmaf_rn((float)cx, p.interval[0], p.cell_xmin[0]);
    const float oy = __fmaf_rn((float)cy, p.interval[1], p.cell_xmin[1]);
    return make_float4(p.domain_xmin[0] - ox, p.domain_xmin[1] - oy, p.domain_xmax[0] - ox, p.domain_xmax[1] - oy);
}

// fluidUpdate (fluid.cu:256-287).  Mixed form: the position offset and the
// velocity are integrated with Kahan compensation.
template <class G, class F> __global__ void __launch_bounds__(kBlock) k_fluid_update(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const int i = blk * blockDim.x + threadIdx.x;
    unsigned int sp2 = 0u, moved2 = 0u;
    if (i < p.fluid_number_total) {
        const int ph = d.f_phase[i];
        const float dt = p.dt;
        float2 x = F::kMixed ? d.f_off[i] : d.f_pos[i], v = d.f_vel[i], a = d.f_dudt[i];
        const float2 x0 = x;
        if (p.transient_type == SPHNJ_STEADY) {
            a.x += -0.1f * v.x;
            a.y += -0.1f * v.y;
            d.f_dudt[i] = a;
        }
        if constexpr (F::kMixed) {
            float2 xc = d.f_offc[i], vc = d.f_velc[i];
            kahan_add2(x, xc, make_float2(v.x * dt, v.y * dt));
            kahan_add2(v, vc, make_float2((a.x + p.gravity[0]) * dt, (a.y + p.gravity[1]) * dt));
            const float4 box = box_in_cell(p, d.f_cell[i]);
            if (x.x < box.x || x.x > box.z) xc.x = 0.0f;
            if (x.y < box.y || x.y > box.w) xc.y = 0.0f;
            x.x = fminf(fmaxf(x.x, box.x), box.z);
            x.y = fminf(fmaxf(x.y, box.y), box.w);
            d.f_off[i] = x;
            d.f_offc[i] = xc;
            d.f_velc[i] = vc;
        } else {
            x.x += v.x * dt;
            x.y += v.y * dt;
            v.x += (a.x + p.gravity[0]) * dt;
            v.y += (a.y + p.gravity[1]) * dt;
            x.x = fminf(fmaxf(x.x, p.domain_xmin[0]), p.domain_xmax[0]);
            x.y = fminf(fmaxf(x.y, p.domain_xmin[1]), p.domain_xmax[1]);
            d.f_pos[i] = x;
        }
        float rho = d.f_rho[i] + d.f_drho[i] * dt;
        rho = fmaxf(rho, by_phase(p.min_density, ph));
        d.f_rho[i] = rho;
        d.f_p[i] = density_to_pressure(p, rho, ph);
        d.f_vel[i] = v;
        if (!(finite2(x) && finite2(v) && isfinite(rho))) raise_error(d.err, SPHNJ_ERR_NONFINITE, KF, i);
        float s2 = __fadd_rn(__fmul_rn(v.x, v.x), __fmul_rn(v.y, v.y));
        if (s2 == s2) sp2 = __float_as_uint(s2);  // NaN never wins, as on the host
        moved2 = disp2(x0, x);
    }
    block_max_to<kBlock>(sp2, d.max_speed2_bits);
    __syncthreads();
    block_max_to<kBlock>(moved2, &d.disp2_bits[0]);
}

// Positions back from the second buffer after an odd number of shifting
// passes (the record's f_x_alt holds them; f_pos / f_off is their home).
template <class G, class F> __global__ void __launch_bounds__(kBlock) k_shift_copy_back(const __grid_constant__ G g) {
    SPHNJ_SCENE(g);
    const int i = blk * blockDim.x + threadIdx.x;
    if (i < p.fluid_number_total) (F::kMixed ? d.f_off : d.f_pos)[i] = d.f_x_alt[i];
}

// staged entries of a tile: three strips of tile_h + 2 cells at per_cell particles
inline int tile_cap(int tile_h, int per_cell = kMaxPerCell) { return 3 * (tile_h + 2) * per_cell; }
inline unsigned tile_blocks(const sphnj_params &p, int tile_h) {
    return (unsigned)p.cell_number[0] * (unsigned)((p.cell_number[1] + tile_h - 1) / tile_h);
}
// Blocks of the tiled sweeps of one scene: about one per tile that the
// scene's fluid can fill at ~8 particles per cell, at most one per tile;
// blocks loop over the active tiles, so a scene whose fluid spreads over more
// tiles than this is still swept in full.
inline unsigned sweep_blocks(const sphnj_params &p, int tile_h) {
    const int nf = p.fluid_number_total;
    if (nf <= 0) return 0u;
    if (!sweep_compacted(p, tile_h)) return tile_blocks(p, tile_h);  // one block per tile
    const long want = std::max<long>(1, ((long)nf + 8L * tile_h - 1) / (8L * tile_h));
    return (unsigned)std::min<long>(tile_blocks(p, tile_h), want);
}
constexpr size_t kPairSmemPerEntry = 3 * sizeof(float2) + sizeof(int) + 1;

}  // namespace

// Every pair-pass instantiation may stage up to kMaxPerCell particles per
// cell of the tallest tile (64 cells): its dynamic shared memory above 48 KB
// needs an opt-in, given once for the largest size.
template <class D, class F, bool kList, int kT, int kMin> cudaError_t allow_pair_smem() {
    const size_t smem = tile_cap(64, kMaxPerCell) * kPairSmemPerEntry;
    return cudaFuncSetAttribute((const void *)k_fluid_pair_tiled<D, F, kList, kT, kMin>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}
template <class D, class G, class F, bool kList> cudaError_t allow_pair_smem_all() {
    using Sh = PairShape<G, kList, F>;
    cudaError_t e = allow_pair_smem<D, F, kList, Sh::threads, Sh::min_blocks>();
    if (e == cudaSuccess) e = allow_pair_smem<D, F, kList, 128, PairBlock<F, kList, 128>::min_blocks>();
    if (e == cudaSuccess) e = allow_pair_smem<D, F, kList, 256, PairBlock<F, kList, 256>::min_blocks>();
    return e;
}

cudaError_t configure_sweeps(const TileConfig &) {
    cudaError_t e = allow_pair_smem_all<One, GroupOne, FormPlain, false>();
    if (e == cudaSuccess) e = allow_pair_smem_all<One, GroupOne, FormPlain, true>();
    if (e == cudaSuccess) e = allow_pair_smem_all<One, GroupOne, FormMixed, false>();
    if (e == cudaSuccess) e = allow_pair_smem_all<One, GroupOne, FormMixed, true>();
    if (e == cudaSuccess) e = allow_pair_smem_all<Many, GroupMany, FormPlain, true>();
    if (e == cudaSuccess) e = allow_pair_smem_all<Many, GroupMany, FormMixed, true>();
    return e;
}

// Single scenes use the active-tile list when sweep_compacted() selects it;
// batches always do (their scenes share one kernel).
template <class G> bool use_tile_list(const G &g) {
    if constexpr (std::is_same<G, GroupMany>::value) return true;
    else return sweep_compacted(g.s.p, g.s.tile_h);
}
// The tallest tile of the group's scenes (sizes a launch's staging).
inline int max_tile_h(const GroupOne &g) { return g.s.tile_h; }
inline int max_tile_h(const GroupMany &g) {
    int h = 1;
    for (int k = 0; k < g.n; ++k) h = std::max(h, g.h_scenes[k].tile_h);
    return h;
}

// Per-particle fallback grid of one scene (grid-stride; it returns at once
// when every particle is listed, as it is on nearly every step): one block per
// 16k particles, at least 16 and at most 2 per SM.
inline unsigned fallback_blocks(int n) {
    if (n <= 0) return 0u;
    const long b = std::min<long>(kFallbackBlocks, std::max<long>(16, (n + 16383) / 16384));
    return (unsigned)std::min<long>(b, grid_for(n, kPairBlock));
}

namespace {

// The tiled pair pass with block shape Sh: list launches get about one
// block per tile the fluid can fill (twice that at 128 threads), a dense
// scene one block per tile.  Each scene sweeps tiles of its own height.
template <class F, class G, bool kList, class Sh>
int pair_tiled(cudaStream_t st, G &g, int cap, int shift_cap, size_t smem) {
    using D = typename G::Dev;
    const long long key = site_key(SITE_PAIR_TILED, Sh::threads);
    if constexpr (kList)
        return launch(
            g, key,
            [](const Scene &s) {
                return std::min<unsigned>(tile_blocks(s.p, s.tile_h),
                                          sweep_blocks(s.p, s.tile_h) * (kTileBlock / Sh::threads));
            },
            k_fluid_pair_tiled<D, F, true, Sh::threads, Sh::min_blocks>, Sh::threads, smem, st, cap, shift_cap);
    else
        return launch(
            g, key, [](const Scene &s) { return tile_blocks(s.p, s.tile_h); },
            k_fluid_pair_tiled<D, F, false, Sh::threads, Sh::min_blocks>, Sh::threads, smem, st, cap, shift_cap);
}

template <class F, class G, bool kList>
int pair_tiled_shape(cudaStream_t st, G &g, const TileConfig &tc, int cap, int shift_cap) {
    const size_t smem = cap * kPairSmemPerEntry;
    if (tc.pair_block == 128) return pair_tiled<F, G, kList, PairBlock<F, kList, 128>>(st, g, cap, shift_cap, smem);
    if (tc.pair_block == 256) return pair_tiled<F, G, kList, PairBlock<F, kList, 256>>(st, g, cap, shift_cap, smem);
    return pair_tiled<F, G, kList, PairShape<G, kList, F>>(st, g, cap, shift_cap, smem);
}

template <class F, class G> int fluid_pair(cudaStream_t st, G &g, const TileConfig &tc) {
    using D = typename G::Dev;
    if (!tc.tiled)
        return launch(
            g, site_key(SITE_PAIR_EACH), [](const Scene &s) { return grid_for(s.p.fluid_number_total, kPairBlock); },
            k_fluid_pair_each<D, F>, kPairBlock, 0, st, 0);
    const bool list = use_tile_list(g);
    const int cap = tile_cap(max_tile_h(g), pair_per_cell(g, list));
    const int shift_cap = tile_cap(max_tile_h(g));  // the shifting passes' staging (shift_pass)
    // this step's active tiles (the cell lists are final), used by the pair
    // pass and every shifting pass of the step
    int n = launch_tile_compact(st, g, std::is_same<G, GroupMany>::value);
    if (list) {
        n += pair_tiled_shape<F, G, true>(st, g, tc, cap, shift_cap);
    } else if constexpr (!std::is_same<G, GroupMany>::value) {  // batches always sweep their lists
        n += pair_tiled_shape<F, G, false>(st, g, tc, cap, shift_cap);
    }
    n += launch(
        g, site_key(SITE_PAIR_FALLBACK), [](const Scene &s) { return fallback_blocks(s.p.fluid_number_total); },
        k_fluid_pair_each<D, F>, kPairBlock, 0, st, 1);
    return n;
}

template <class F, class G> int fluid_update(cudaStream_t st, G &g) {
    return launch(
        g, site_key(SITE_FLUID_UPDATE), [](const Scene &s) { return grid_for(s.p.fluid_number_total, kBlock); },
        k_fluid_update<typename G::Dev, F>, kBlock, 0, st);
}

// Pass k reads the positions from f_pos / f_off and writes them to f_x_alt;
// odd passes run with the two exchanged, so pass k + 1 reads what pass k
// wrote and the positions are home again after every even pass.
template <class G> struct PositionsExchanged {
    G &g;
    bool on;
    PositionsExchanged(G &g_, bool on_) : g(g_), on(on_) {
        if (on) g.exchange_positions();
    }
    ~PositionsExchanged() {
        if (on) g.exchange_positions();
    }
};

template <class F, class G> int shift_pass(cudaStream_t st, G &g, const TileConfig &tc, int pass) {
    using D = typename G::Dev;
    auto active = [pass](const Scene &s) { return s.p.fluid_number_total > 0 && pass < s.p.shift_per_step; };
    int gathered = 0;
    if (pass == 0)  // the listed particles' positions and cells into list order
        gathered = launch(
            g, site_key(SITE_SHIFT_GATHER),
            [&](const Scene &s) { return active(s) ? grid_for(s.p.fluid_number_total, kBlock) : 0u; },
            k_shift_gather<D, F>, kBlock, 0, st);
    const PositionsExchanged<G> buffers(g, (pass & 1) != 0);
    if (!tc.tiled)
        return gathered +
               launch(
                   g, site_key(SITE_SHIFT_EACH, pass),
                   [&](const Scene &s) { return active(s) ? grid_for(s.p.fluid_number_total, kPairBlock) : 0u; },
                   k_shift_gradient_each<D, F>, kPairBlock, 0, st, 0, pass) +
               launch(
                   g, site_key(SITE_SHIFT_FALLBACK, pass),
                   [&](const Scene &s) { return active(s) ? fallback_blocks(s.p.fluid_number_total) : 0u; },
                   k_shift_gradient_each<D, F>, kPairBlock, 0, st, 1, pass);
    const int cap = tile_cap(max_tile_h(g));  // also the pair pass's shift_cap (fluid_pair)
    const size_t smem = cap * sizeof(float2);
    // batched list launches: blocks of kListBlock threads, kTileBlock / kListBlock
    // times as many (a sparse scene swept alone, one short launch, keeps the
    // larger blocks: measured 116 against 132 ms/step on the sweep's scenes
    // stepped one by one).  A dense scene: one block of kDenseBlock threads
    // per tile (4.15M dam break 3.92 -> 3.80 ms/step against 256 threads;
    // 64 threads: 4.39, 512: 4.73).  tc.shift_block overrides either.
    constexpr int kDefaultList = std::is_same<G, GroupMany>::value ? kListBlock : kTileBlock;
    const bool list = use_tile_list(g);
    const int kT = tc.shift_block ? tc.shift_block : list ? kDefaultList : kDenseBlock;
    const long long key = site_key(SITE_SHIFT_TILED, (kT << 8) | pass);
    auto go = [&](auto threads) {
        constexpr int T = decltype(threads)::value;
        if (list)
            return launch(
                g, key,
                [&](const Scene &s) {
                    return active(s) ? std::min<unsigned>(tile_blocks(s.p, s.tile_h),
                                                          sweep_blocks(s.p, s.tile_h) * std::max(1, kTileBlock / T))
                                     : 0u;
                },
                k_shift_gradient_tiled<D, F, true, T>, T, smem, st, cap, pass);
        return launch(
            g, key, [&](const Scene &s) { return active(s) ? sweep_blocks(s.p, s.tile_h) : 0u; },
            k_shift_gradient_tiled<D, F, false, T>, T, smem, st, cap, pass);
    };
    int n = kT == 64 ? go(std::integral_constant<int, 64>{})
            : kT == 256 ? go(std::integral_constant<int, 256>{})
                        : go(std::integral_constant<int, 128>{});
    n += launch(
        g, site_key(SITE_SHIFT_FALLBACK, pass),
        [&](const Scene &s) { return active(s) ? fallback_blocks(s.p.fluid_number_total) : 0u; },
        k_shift_gradient_each<D, F>, kPairBlock, 0, st, 1, pass);
    return gathered + n;
}

// After the last pass: the unlisted particles' positions back from f_x_alt
// after an odd number of passes (every particle is copied; the listed ones
// are overwritten next), then the listed ones from list order.
template <class F, class G> int shift_copy_back(cudaStream_t st, G &g) {
    int n = launch(
        g, site_key(SITE_SHIFT_COPY_BACK),
        [](const Scene &s) { return (s.p.shift_per_step & 1) ? grid_for(s.p.fluid_number_total, kBlock) : 0u; },
        k_shift_copy_back<typename G::Dev, F>, kBlock, 0, st);
    n += launch(
        g, site_key(SITE_SHIFT_SCATTER),
        [](const Scene &s) {
            return s.p.fluid_number_total > 0 && s.p.shift_per_step > 0 ? grid_for(s.p.fluid_number_total, kBlock)
                                                                        : 0u;
        },
        k_shift_scatter<typename G::Dev, F>, kBlock, 0, st);
    return n;
}

}  // namespace

template <class G> int launch_fluid_pair(cudaStream_t st, G &g, const TileConfig &tc) {
    return g.form == SPHNJ_FORM_MIXED ? fluid_pair<FormMixed>(st, g, tc) : fluid_pair<FormPlain>(st, g, tc);
}
template <class G> int launch_fluid_update(cudaStream_t st, G &g) {
    return g.form == SPHNJ_FORM_MIXED ? fluid_update<FormMixed>(st, g) : fluid_update<FormPlain>(st, g);
}
template <class G> int launch_shift_pass(cudaStream_t st, G &g, const TileConfig &tc, int pass) {
    return g.form == SPHNJ_FORM_MIXED ? shift_pass<FormMixed>(st, g, tc, pass) : shift_pass<FormPlain>(st, g, tc, pass);
}
template <class G> int launch_shift_copy_back(cudaStream_t st, G &g) {
    return g.form == SPHNJ_FORM_MIXED ? shift_copy_back<FormMixed>(st, g) : shift_copy_back<FormPlain>(st, g);
}

SPHNJ_INSTANTIATE_GROUPS(launch_fluid_pair, const TileConfig &);
SPHNJ_INSTANTIATE_GROUPS(launch_fluid_update);
SPHNJ_INSTANTIATE_GROUPS(launch_shift_pass, const TileConfig &, int);
SPHNJ_INSTANTIATE_GROUPS(launch_shift_copy_back);

}  // namespace sphnj
