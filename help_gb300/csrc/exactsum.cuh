// Exact sums of doubles on the integer pipes.
//
// GB300 issues FP64 at ~2 lanes per clock per SM: an FP64 warp instruction
// holds its sub-partition's pipe ~64 cycles however few lanes are active, so
// every level of an FP64 reduction tree costs that much on the critical path.
// These sums align the values on their largest exponent into 128-bit
// two's-complement fixed point (integer shuffles and adds, no FP64 pipe),
// add them exactly, and round once to the nearest double (ties to even).
// The result does not depend on the order of the additions -- every thread
// and every CTA that sums the same values gets the same bits -- and is at
// least as accurate as any summation order in FP64.
//
// Alignment: the largest value's leading bit sits at bit 116 of the
// accumulator (53-bit significand shifted left by 64), leaving 10 bits of
// headroom for up to 1,024 terms.  A term more than 2^-64 below the largest
// term's least significant bit loses its low bits (an error below 2^-117 of
// the largest term).  Non-finite inputs are not aligned: the callers fall
// back to an FP64 sum, which propagates NaN / Inf.
#pragma once

#include "common.cuh"

namespace help {

struct Fixed128 {
    unsigned long long lo, hi;
};

HELP_DEVINL void add_fixed(Fixed128& a, const Fixed128& b) {
    const unsigned long long lo = a.lo + b.lo;
    a.hi = a.hi + b.hi + (lo < a.lo ? 1ull : 0ull);
    a.lo = lo;
}

// Alignment exponent of v: the biased exponent field, 1 for subnormals (their
// scale), 0 for zero, 2047 for Inf / NaN.
HELP_DEVINL int exact_exp(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7ff);
    return e != 0 ? e : ((b << 1) != 0 ? 1 : 0);
}

// v as a fixed-point integer whose unit is 2^(emax - 1075 - 64) (emax >= the
// alignment exponent of v, finite v).
HELP_DEVINL Fixed128 to_fixed(double v, int emax) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7ff);
    unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    int ee = 1;
    if (e != 0) {
        m |= 1ull << 52;
        ee = e;
    }
    const int sh = ee - emax + 64;  // <= 64
    Fixed128 r = {0ull, 0ull};
    if (m != 0 && sh > -53) {
        if (sh < 0) {
            r.lo = m >> (-sh);
        } else if (sh == 0) {
            r.lo = m;
        } else if (sh < 64) {
            r.lo = m << sh;
            r.hi = m >> (64 - sh);
        } else {
            r.hi = m;
        }
    }
    if (b >> 63) {  // negate
        r.lo = ~r.lo;
        r.hi = ~r.hi;
        if (++r.lo == 0) ++r.hi;
    }
    return r;
}

// The double nearest (ties to even) to s * 2^(emax - 1075 - 64).
HELP_DEVINL double from_fixed(Fixed128 s, int emax) {
    const bool neg = (long long)s.hi < 0;
    if (neg) {
        s.lo = ~s.lo;
        s.hi = ~s.hi;
        if (++s.lo == 0) ++s.hi;
    }
    if (s.hi == 0 && s.lo == 0) return 0.0;
    const int lz = s.hi ? __clzll((long long)s.hi) : 64 + __clzll((long long)s.lo);
    unsigned long long top, rest;
    if (lz >= 64) {
        top = s.lo << (lz - 64);
        rest = 0;
    } else if (lz == 0) {
        top = s.hi;
        rest = s.lo;
    } else {
        top = (s.hi << lz) | (s.lo >> (64 - lz));
        rest = s.lo << lz;
    }
    if (rest != 0) top |= 1ull;  // sticky: the 11 bits below the double's last keep it
    const double d = __ull2double_rn(top);  // top in [2^63, 2^64)
    const int k = emax - 1075 - lz;       // value = top * 2^k
    double r;
    if (k >= -1022 && k <= 1023) r = d * __longlong_as_double((long long)(k + 1023) << 52);
    else r = scalbn(d, k);
    return neg ? -r : r;
}

// Butterfly over groups of W lanes (W a power of two <= 32): every lane of a
// group ends with the group's total.
template <int W>
HELP_DEVINL int group_max_int(int v) {
#pragma unroll
    for (int o = W >> 1; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
template <int W>
HELP_DEVINL Fixed128 group_add_fixed(Fixed128 a) {
#pragma unroll
    for (int o = W >> 1; o > 0; o >>= 1) {
        Fixed128 b;
        b.lo = __shfl_xor_sync(0xffffffffu, a.lo, o);
        b.hi = __shfl_xor_sync(0xffffffffu, a.hi, o);
        add_fixed(a, b);
    }
    return a;
}

// Exact sum over each group of W lanes of the lanes' values (up to N per
// lane, unused slots 0.0).  Identical in every lane of a group.  Call with
// the whole warp converged; the control flow stays warp-uniform (the groups
// of a warp shuffle together), so a group of zeros runs the same
// instructions (its total comes out 0).
template <int W, int N>
HELP_DEVINL double group_sum_exact(const double (&v)[N]) {
    int e = 0;
#pragma unroll
    for (int i = 0; i < N; ++i) e = max(e, exact_exp(v[i]));
    e = group_max_int<W>(e);
    if (__any_sync(0xffffffffu, e == 2047)) {  // Inf or NaN in the warp: FP64 sums propagate them
        double s = 0.0;
#pragma unroll
        for (int i = 0; i < N; ++i) s += v[i];
#pragma unroll
        for (int o = W >> 1; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        return s;
    }
    Fixed128 a = {0ull, 0ull};
#pragma unroll
    for (int i = 0; i < N; ++i) add_fixed(a, to_fixed(v[i], e));
    return from_fixed(group_add_fixed<W>(a), e);  // 0.0 for a group of zeros
}
template <int W>
HELP_DEVINL double group_sum_exact(double v) {
    const double a[1] = {v};
    return group_sum_exact<W, 1>(a);
}

// Scratch of the block sums: per warp, two exponents and two partials.
struct ExactScratch {
    int emax[2][32];
    Fixed128 part[2][32];
};

// Exact sums over the whole CTA of u and v (one of each per thread); every
// thread gets both totals.  Three __syncthreads.
HELP_DEVINL void block_sum2_exact(double& u, double& v, ExactScratch* s) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int eu = __reduce_max_sync(0xffffffffu, (unsigned)exact_exp(u));
    const int ev = __reduce_max_sync(0xffffffffu, (unsigned)exact_exp(v));
    __syncthreads();  // the previous call's readers are done with s
    if (lane == 0) {
        s->emax[0][warp] = eu;
        s->emax[1][warp] = ev;
    }
    __syncthreads();
    int mu = 0, mv = 0;
    for (int w = 0; w < nw; ++w) {
        mu = max(mu, s->emax[0][w]);
        mv = max(mv, s->emax[1][w]);
    }
    // the block-uniform fallback for non-finite values: plain FP64 sums
    if (mu == 2047 || mv == 2047) {
        double a = u, b = v;
        a = warp_sum(a);
        b = warp_sum(b);
        if (lane == 0) {
            s->part[0][warp].lo = (unsigned long long)__double_as_longlong(a);
            s->part[1][warp].lo = (unsigned long long)__double_as_longlong(b);
        }
        __syncthreads();
        a = 0.0;
        b = 0.0;
        for (int w = 0; w < nw; ++w) {
            a += __longlong_as_double((long long)s->part[0][w].lo);
            b += __longlong_as_double((long long)s->part[1][w].lo);
        }
        u = a;
        v = b;
        return;
    }
    const Fixed128 fu = group_add_fixed<32>(to_fixed(u, mu));  // zeros when mu == 0
    const Fixed128 fv = group_add_fixed<32>(to_fixed(v, mv));
    if (lane == 0) {
        s->part[0][warp] = fu;
        s->part[1][warp] = fv;
    }
    __syncthreads();
    Fixed128 tu = {0ull, 0ull}, tv = {0ull, 0ull};
    for (int w = 0; w < nw; ++w) {
        add_fixed(tu, s->part[0][w]);
        add_fixed(tv, s->part[1][w]);
    }
    u = from_fixed(tu, mu);
    v = from_fixed(tv, mv);
}

HELP_DEVINL double block_sum_exact(double u, ExactScratch* s) {
    double v = 0.0;
    block_sum2_exact(u, v, s);
    return u;
}

}  // namespace help
