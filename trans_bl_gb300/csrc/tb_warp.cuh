// tb_warp.cuh -- second-order linear recurrences along a line shared by the
// 32 lanes of a warp.
//
// The x-direction solves of the stage (pentadiagonal LU sweeps, the 4th-order
// implicit x integrations of continuity and of the wall vorticity) are
// recurrences y_i = f(y_{i-1}, y_{i-2}) along lines of ~1000 points.  One
// thread per line leaves most of the GPU idle (a few hundred lines); here a
// warp owns a line and lane t owns rows [r0, r1) = [tS, min(n, tS + S)).  A
// recurrence runs in three passes:
//   1. local pass with zero carry-in, plus the chunk's 2x2 transfer matrix
//      (responses of its last two rows to unit carries);
//   2. Kogge-Stone scan of (transfer matrix, local end state) over the lanes,
//      which gives every lane the true values of the two rows before it;
//   3. fix-up: the homogeneous recurrence started from those carries, added.
// Rows live in shared memory in lane chunks: row i at (i / S) * Sp + i % S,
// Sp = S rounded up to odd so that 16-byte accesses at equal chunk offsets
// of 8 consecutive lanes fall in distinct banks.
#pragma once
#include "tb_internal.h"

struct WarpLine {
    int n, S, Sp;
    __device__ __forceinline__ int slot(int i) const { return (i / S) * Sp + i % S; }
    static __host__ __device__ int chunk(int n) { return (n + 31) / 32; }
    static __host__ __device__ int padded(int n) { return chunk(n) | 1; }
};

// Forward: y_i = v_i - a(i) y_{i-1} - b(i) y_{i-2} for all rows of the line,
// y_{-1} = y_{-2} = 0.  Bl holds this lane's rows (v on entry, y on exit).
template <class FA, class FB>
__device__ __forceinline__ void warp_rec2_fwd(cplx* Bl, int r0, int r1, int lane, FA a, FB b) {
    cplx y1 = make_double2(0.0, 0.0), y2 = make_double2(0.0, 0.0);
    double p1 = 1.0, p2 = 0.0, q1 = 0.0, q2 = 1.0;   // responses to carries (y_{r0-1}, y_{r0-2}) = (1,0), (0,1)
    for (int i = r0; i < r1; i++) {
        double ai = a(i), bi = b(i);
        cplx v = Bl[i - r0];
        cplx y = make_double2(v.x - ai * y1.x - bi * y2.x, v.y - ai * y1.y - bi * y2.y);
        Bl[i - r0] = y;
        y2 = y1; y1 = y;
        double p = -ai * p1 - bi * p2; p2 = p1; p1 = p;
        double q = -ai * q1 - bi * q2; q2 = q1; q1 = q;
    }
    // end state E = M C + e with C the carries, M = [[p1, q1], [p2, q2]], e = (y1, y2)
    double m00 = p1, m01 = q1, m10 = p2, m11 = q2;
    cplx e0 = y1, e1 = y2;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        double n00 = __shfl_up_sync(0xffffffffu, m00, off), n01 = __shfl_up_sync(0xffffffffu, m01, off);
        double n10 = __shfl_up_sync(0xffffffffu, m10, off), n11 = __shfl_up_sync(0xffffffffu, m11, off);
        cplx f0, f1;
        f0.x = __shfl_up_sync(0xffffffffu, e0.x, off); f0.y = __shfl_up_sync(0xffffffffu, e0.y, off);
        f1.x = __shfl_up_sync(0xffffffffu, e1.x, off); f1.y = __shfl_up_sync(0xffffffffu, e1.y, off);
        if (lane >= off) {
            // compose: E_t = M_t (M_s C_s + e_s) + e_t
            e0 = make_double2(e0.x + m00 * f0.x + m01 * f1.x, e0.y + m00 * f0.y + m01 * f1.y);
            e1 = make_double2(e1.x + m10 * f0.x + m11 * f1.x, e1.y + m10 * f0.y + m11 * f1.y);
            double t00 = m00 * n00 + m01 * n10, t01 = m00 * n01 + m01 * n11;
            double t10 = m10 * n00 + m11 * n10, t11 = m10 * n01 + m11 * n11;
            m00 = t00; m01 = t01; m10 = t10; m11 = t11;
        }
    }
    cplx c1, c2;   // true y_{r0-1}, y_{r0-2}
    c1.x = __shfl_up_sync(0xffffffffu, e0.x, 1); c1.y = __shfl_up_sync(0xffffffffu, e0.y, 1);
    c2.x = __shfl_up_sync(0xffffffffu, e1.x, 1); c2.y = __shfl_up_sync(0xffffffffu, e1.y, 1);
    if (lane == 0) { c1 = make_double2(0.0, 0.0); c2 = c1; }
    for (int i = r0; i < r1; i++) {
        double ai = a(i), bi = b(i);
        cplx z = make_double2(-ai * c1.x - bi * c2.x, -ai * c1.y - bi * c2.y);
        c2 = c1; c1 = z;
        cplx y = Bl[i - r0];
        Bl[i - r0] = make_double2(y.x + z.x, y.y + z.y);
    }
}

// Backward: x_i = (y_i - c(i) x_{i+1} - d(i) x_{i+2}) * s(i) for all rows,
// x_n = x_{n+1} = 0.  Bl holds this lane's rows (y on entry, x on exit).
template <class FC, class FD, class FS>
__device__ __forceinline__ void warp_rec2_bwd(cplx* Bl, int r0, int r1, int lane, FC c, FD d, FS s) {
    cplx x1 = make_double2(0.0, 0.0), x2 = make_double2(0.0, 0.0);
    double p1 = 1.0, p2 = 0.0, q1 = 0.0, q2 = 1.0;   // responses to (x_{r1}, x_{r1+1})
    for (int i = r1 - 1; i >= r0; i--) {
        double ci = c(i), di = d(i), si = s(i);
        cplx y = Bl[i - r0];
        cplx x = make_double2((y.x - ci * x1.x - di * x2.x) * si, (y.y - ci * x1.y - di * x2.y) * si);
        Bl[i - r0] = x;
        x2 = x1; x1 = x;
        double p = (-ci * p1 - di * p2) * si; p2 = p1; p1 = p;
        double q = (-ci * q1 - di * q2) * si; q2 = q1; q1 = q;
    }
    double m00 = p1, m01 = q1, m10 = p2, m11 = q2;
    cplx e0 = x1, e1 = x2;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        double n00 = __shfl_down_sync(0xffffffffu, m00, off), n01 = __shfl_down_sync(0xffffffffu, m01, off);
        double n10 = __shfl_down_sync(0xffffffffu, m10, off), n11 = __shfl_down_sync(0xffffffffu, m11, off);
        cplx f0, f1;
        f0.x = __shfl_down_sync(0xffffffffu, e0.x, off); f0.y = __shfl_down_sync(0xffffffffu, e0.y, off);
        f1.x = __shfl_down_sync(0xffffffffu, e1.x, off); f1.y = __shfl_down_sync(0xffffffffu, e1.y, off);
        if (lane + off < 32) {
            e0 = make_double2(e0.x + m00 * f0.x + m01 * f1.x, e0.y + m00 * f0.y + m01 * f1.y);
            e1 = make_double2(e1.x + m10 * f0.x + m11 * f1.x, e1.y + m10 * f0.y + m11 * f1.y);
            double t00 = m00 * n00 + m01 * n10, t01 = m00 * n01 + m01 * n11;
            double t10 = m10 * n00 + m11 * n10, t11 = m10 * n01 + m11 * n11;
            m00 = t00; m01 = t01; m10 = t10; m11 = t11;
        }
    }
    cplx c1, c2;   // true x_{r1}, x_{r1+1}
    c1.x = __shfl_down_sync(0xffffffffu, e0.x, 1); c1.y = __shfl_down_sync(0xffffffffu, e0.y, 1);
    c2.x = __shfl_down_sync(0xffffffffu, e1.x, 1); c2.y = __shfl_down_sync(0xffffffffu, e1.y, 1);
    if (lane == 31) { c1 = make_double2(0.0, 0.0); c2 = c1; }
    for (int i = r1 - 1; i >= r0; i--) {
        double ci = c(i), di = d(i), si = s(i);
        cplx z = make_double2((-ci * c1.x - di * c2.x) * si, (-ci * c1.y - di * c2.y) * si);
        c2 = c1; c1 = z;
        cplx x = Bl[i - r0];
        Bl[i - r0] = make_double2(x.x + z.x, x.y + z.y);
    }
}
