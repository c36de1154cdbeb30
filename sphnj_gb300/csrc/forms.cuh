// The two forms of the method, as the neighbour loops see them.
//
// FormPlain  the reference's precision (include/types.h): fluid and virtual
//            positions absolute FP32, solid state FP64.  Pair vectors are
//            differences of absolute positions, exactly as the reference
//            forms them.
// FormMixed  positions are an integer cell plus an FP32 offset from the
//            cell's lower-left corner.  A neighbour loop works in the frame
//            of one cell (the home particle's own cell, or the origin of a
//            tile): a particle listed in cell m sits at
//                (m - frame) * cell width + its offset,
//            which keeps ~eps * (a few cell widths) of absolute precision
//            anywhere in the domain instead of eps * |x|.
#pragma once

#include "device_common.cuh"

namespace sphnj {

__device__ __forceinline__ float2 add2(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }

// Frame arithmetic of the mixed form is written with round-to-nearest
// intrinsics: a frame shift k * width is loop-invariant in the neighbour
// loops, and left to the compiler it may be hoisted (two roundings) in one
// instantiation of a kernel and contracted into an FMA with the offset (one
// rounding) in another - the one-scene and batched launches would then
// differ in the last bit.
__device__ __forceinline__ float2 add2_rn(float2 a, float2 b) {
    return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y));
}
__device__ __forceinline__ float2 cells_to_len(const sphnj_params &p, int kx, int ky) {
    return make_float2(__fmul_rn((float)kx, p.interval[0]), __fmul_rn((float)ky, p.interval[1]));
}

// Packed FP32 pairs (PTX .f32x2 on sm_100 and later): one instruction does
// the same two round-to-nearest operations as two scalar ones (same
// results), on the x and y halves of a float2.  The mixed form's pair and
// shifting loops use them for their vector arithmetic.
__device__ __forceinline__ float2 sub2x(float2 a, float2 b) {
    float2 r;
    asm("{\n\t.reg .b64 a, b, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\t"
        "sub.rn.f32x2 d, a, b;\n\tmov.b64 {%0, %1}, d;\n\t}"
        : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ float2 mul2x(float2 a, float2 b) {
    float2 r;
    asm("{\n\t.reg .b64 a, b, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\t"
        "mul.rn.f32x2 d, a, b;\n\tmov.b64 {%0, %1}, d;\n\t}"
        : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
// a * b + c per half, each one fused multiply-add
__device__ __forceinline__ float2 fma2x(float2 a, float2 b, float2 c) {
    float2 r;
    asm("{\n\t.reg .b64 a, b, c, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\t"
        "mov.b64 c, {%6, %7};\n\tfma.rn.f32x2 d, a, b, c;\n\tmov.b64 {%0, %1}, d;\n\t}"
        : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return r;
}
__device__ __forceinline__ float2 splat2(float a) { return make_float2(a, a); }

// 2^x by the SFU (PTX ex2.approx.ftz.f32, relative error ~2^-22)
__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Gaussian kernel-gradient factor W'(r) = exp(-r^2 / h^2) Kd C32 (fluid.cu:44-46)
// from r^2, as each form evaluates it: the plain form keeps the reference's
// expression and rounding (exp of -q^2, then times Kd, then times C32); the
// mixed form folds the constants, 2^(r^2 a) b with a = -log2(e) / h^2 and
// b = Kd C32 (both loop-invariant), one multiply, one SFU op, one multiply.
__device__ __forceinline__ float gw_plain(const sphnj_params &p, float r2) {
    return __expf(-(r2 * p.smoothing_length_inverse_square)) * p.kernel_differential * p.coefficient_3d_to_2d;
}
__device__ __forceinline__ float gw_folded(const sphnj_params &p, float r2) {
    const float a = -1.4426950408889634f * p.smoothing_length_inverse_square;
    const float b = p.kernel_differential * p.coefficient_3d_to_2d;
    return ex2_approx(r2 * a) * b;
}

// Home cell minus frame cell, in cells (mixed form; ignored by the plain form).
struct Frame {
    int dx, dy;
};

struct FormPlain {
    static constexpr bool kMixed = false;
    __device__ static __forceinline__ float gw(const sphnj_params &p, float r2) { return gw_plain(p, r2); }
    // shifting gradient: the reference's per-pair weight, no factor after the sum
    static constexpr bool kShiftScaled = false;
    __device__ static __forceinline__ float gw_shift(const sphnj_params &p, float r2) { return gw_plain(p, r2); }
    __device__ static __forceinline__ float shift_scale(const sphnj_params &) { return 1.0f; }
    // frame shift of neighbour slot n (0..8) of the home cell
    __device__ static __forceinline__ float2 shift(const sphnj_params &, Frame, int) { return make_float2(0.f, 0.f); }
    __device__ static __forceinline__ float2 f_home(const sphnj_params &, const DevState &d, Frame, int i) {
        return d.f_pos[i];
    }
    __device__ static __forceinline__ float2 f_nbr(const DevState &d, int j, float2) { return __ldg(&d.f_pos[j]); }
    // the shifting passes' list-order positions, by CSR position h
    __device__ static __forceinline__ float2 f_home_l(const sphnj_params &, const DevState &d, Frame, int h) {
        return d.f_xl[h];
    }
    __device__ static __forceinline__ float2 f_nbr_l(const DevState &d, int t, float2) { return __ldg(&d.f_xl[t]); }
    __device__ static __forceinline__ float2 s_home(const sphnj_params &, const DevState &d, Frame, int i) {
        return to_f2(d.s_pos[i]);
    }
    __device__ static __forceinline__ float2 s_nbr(const DevState &d, int j, float2) { return to_f2(d.s_pos[j]); }
    __device__ static __forceinline__ float2 s_vel(const DevState &d, int j) { return to_f2(d.s_vel[j]); }
    __device__ static __forceinline__ float2 v_home(const sphnj_params &, const DevState &d, Frame, int i) {
        return d.v_pos[i];
    }
    __device__ static __forceinline__ float2 v_nbr(const DevState &d, int j, float2) { return __ldg(&d.v_pos[j]); }
};

struct FormMixed {
    static constexpr bool kMixed = true;
    __device__ static __forceinline__ float gw(const sphnj_params &p, float r2) { return gw_folded(p, r2); }
    // shifting gradient: sum dx 2^(r^2 a) per pair, times b = Kd C32 once
    // for the finished sum (one multiply per pair fewer)
    static constexpr bool kShiftScaled = true;
    __device__ static __forceinline__ float gw_shift(const sphnj_params &p, float r2) {
        return ex2_approx(r2 * (-1.4426950408889634f * p.smoothing_length_inverse_square));
    }
    __device__ static __forceinline__ float shift_scale(const sphnj_params &p) {
        return p.kernel_differential * p.coefficient_3d_to_2d;
    }
    __device__ static __forceinline__ float2 shift(const sphnj_params &p, Frame f, int n) {
        return cells_to_len(p, f.dx + n / 3 - 1, f.dy + n % 3 - 1);
    }
    __device__ static __forceinline__ float2 corner(const sphnj_params &p, Frame f) {
        return cells_to_len(p, f.dx, f.dy);
    }
    __device__ static __forceinline__ float2 f_home(const sphnj_params &p, const DevState &d, Frame f, int i) {
        return add2_rn(d.f_off[i], corner(p, f));
    }
    __device__ static __forceinline__ float2 f_nbr(const DevState &d, int j, float2 sh) {
        return add2_rn(__ldg(&d.f_off[j]), sh);
    }
    __device__ static __forceinline__ float2 f_home_l(const sphnj_params &p, const DevState &d, Frame f, int h) {
        return add2_rn(d.f_xl[h], corner(p, f));
    }
    __device__ static __forceinline__ float2 f_nbr_l(const DevState &d, int t, float2 sh) {
        return add2_rn(__ldg(&d.f_xl[t]), sh);
    }
    __device__ static __forceinline__ float2 s_home(const sphnj_params &p, const DevState &d, Frame f, int i) {
        return add2_rn(d.s_off[i], corner(p, f));
    }
    __device__ static __forceinline__ float2 s_nbr(const DevState &d, int j, float2 sh) {
        return add2_rn(__ldg(&d.s_off[j]), sh);
    }
    __device__ static __forceinline__ float2 s_vel(const DevState &d, int j) { return __ldg(&d.s_v[j]); }
    __device__ static __forceinline__ float2 v_home(const sphnj_params &p, const DevState &d, Frame f, int i) {
        return add2_rn(d.v_off[i], corner(p, f));
    }
    __device__ static __forceinline__ float2 v_nbr(const DevState &d, int j, float2 sh) {
        return add2_rn(__ldg(&d.v_off[j]), sh);
    }
};

// Current position of a solid particle relative to the corner of cell c:
// its reference offset plus displacement, shifted by (reference cell - c).
// Binning and every solid sub-step write it, so the neighbour loops of the
// rest of the step see the solid where it is now.
__device__ __forceinline__ float2 solid_offset(const sphnj_params &p, int2 rc, float2 roff, float2 u, int c) {
    const int ny = p.cell_number[1];
    const int cx = c / ny, cy = c - cx * ny;
    return add2_rn(add2_rn(roff, u), cells_to_len(p, rc.x - cx, rc.y - cy));
}

// Kahan-compensated accumulation x += y with compensation c (Kahan 1965,
// "Further remarks on reducing truncation errors"): c carries the low-order
// part lost by the last addition.
__device__ __forceinline__ void kahan_add(float &x, float &c, float y) {
    const float yc = __fsub_rn(y, c);
    const float t = __fadd_rn(x, yc);
    c = __fsub_rn(__fsub_rn(t, x), yc);
    x = t;
}
__device__ __forceinline__ void kahan_add2(float2 &x, float2 &c, float2 y) {
    kahan_add(x.x, c.x, y.x);
    kahan_add(x.y, c.y, y.y);
}

}  // namespace sphnj
