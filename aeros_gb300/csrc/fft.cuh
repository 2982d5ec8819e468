// fft.cuh -- shared-memory mixed-radix (4, 2, 3, 5) Stockham FFT in FP64.
//
// Replaces FFTW's longitude transforms inside SHTns.  A real row of length
// nlon is transformed as a complex sequence of n = nlon/2 points (even/odd
// samples packed into re/im) plus an O(n) untangling pass.  Rows of one CTA
// are transformed together; each stage ping-pongs between two shared buffers
// (autosort, no bit reversal).  Stage of radix R with running size Ns:
//   v_r = x[j + r n/R] * w^{(j mod Ns) r n/(Ns R)},  v <- DFT_R(v),
//   y[(j - j mod Ns) R + j mod Ns + r Ns] = v_r.
#pragma once
#include "aeros_internal.h"
#include "df.cuh"

namespace aeros {

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cmulconj(double2 a, double2 b) {  // a * conj(b)
    return make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
// multiply by -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ double2 rot90(double2 a) {
    return INV ? make_double2(-a.y, a.x) : make_double2(a.y, -a.x);
}

// Small DFTs, sign -1 (forward) or +1 (INV).  Constants are cos/sin of 2 pi k/R.
template <int R, bool INV>
__device__ __forceinline__ void dft_small(double2 *v) {
    if constexpr (R == 2) {
        double2 a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    } else if constexpr (R == 4) {
        double2 a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
        double2 a2 = cadd(v[1], v[3]), a3 = rot90<INV>(csub(v[1], v[3]));
        v[0] = cadd(a0, a2);
        v[2] = csub(a0, a2);
        v[1] = cadd(a1, a3);
        v[3] = csub(a1, a3);
    } else if constexpr (R == 3) {
        const double c1 = -0.5, s1 = 0.86602540378443864676;
        double2 t1 = cadd(v[1], v[2]), t2 = csub(v[1], v[2]);
        double2 b = make_double2(v[0].x + c1 * t1.x, v[0].y + c1 * t1.y);
        double2 r = rot90<INV>(cscale(t2, s1));
        v[0] = cadd(v[0], t1);
        v[1] = cadd(b, r);
        v[2] = csub(b, r);
    } else if constexpr (R == 5) {
        const double c1 = 0.30901699437494742410, c2 = -0.80901699437494742410;
        const double s1 = 0.95105651629515357212, s2 = 0.58778525229247312917;
        double2 t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
        double2 t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
        double2 b1 = make_double2(v[0].x + c1 * t1.x + c2 * t2.x, v[0].y + c1 * t1.y + c2 * t2.y);
        double2 b2 = make_double2(v[0].x + c2 * t1.x + c1 * t2.x, v[0].y + c2 * t1.y + c1 * t2.y);
        double2 r1 = rot90<INV>(make_double2(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y));
        double2 r2 = rot90<INV>(make_double2(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y));
        v[0] = cadd(v[0], cadd(t1, t2));
        v[1] = cadd(b1, r1);
        v[4] = csub(b1, r1);
        v[2] = cadd(b2, r2);
        v[3] = csub(b2, r2);
    }
}

// Row layout in shared memory: complex element i of a row sits at fpad(i) =
// i + i/8, one spare slot after every 8 values, so that the strided writes of
// a stage (stride R at Ns = 1, R^2 at Ns = R) spread over all 32 banks instead
// of two or four; a row of n values takes frow(n) = n + n/8 slots (n is a
// multiple of 8 for every grid here).
__host__ __device__ constexpr int frow(int n) { return n + n / 8; }
__device__ __forceinline__ int fpad(int i) { return i + (i >> 3); }

// The same small DFTs in double-float (the split form's transforms on the FP32
// pipes); the constants are the nearest double-floats of cos and sin of 2 pi k/R.
template <int R, bool INV>
__device__ __forceinline__ void dft_small(dfc *v) {
    if constexpr (R == 2) {
        dfc a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    } else if constexpr (R == 4) {
        dfc a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
        dfc a2 = cadd(v[1], v[3]), a3 = rot90<INV>(csub(v[1], v[3]));
        v[0] = cadd(a0, a2);
        v[2] = csub(a0, a2);
        v[1] = cadd(a1, a3);
        v[3] = csub(a1, a3);
    } else if constexpr (R == 3) {
        const df2 s1{0x1.bb67aep-1f, 0x1.0b0996p-26f};   // sin(2 pi / 3)
        dfc t1 = cadd(v[1], v[2]), t2 = csub(v[1], v[2]);
        dfc b = csub(v[0], dfc{df_scale(t1.r, 0.5f), df_scale(t1.i, 0.5f)});   // v0 + cos(2 pi/3) t1
        dfc r = rot90<INV>(cscale(t2, s1));
        v[0] = cadd(v[0], t1);
        v[1] = cadd(b, r);
        v[2] = csub(b, r);
    } else if constexpr (R == 5) {
        const df2 c1{0x1.3c6ef4p-2f, -0x1.1a02d6p-27f}, c2{-0x1.9e377ap-1f, 0x1.1a02d6p-27f};
        const df2 s1{0x1.e6f0e2p-1f, -0x1.97756p-26f}, s2{0x1.2cf23p-1f, 0x1.1d5698p-27f};
        dfc t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
        dfc t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
        dfc b1 = cadd(v[0], cadd(cscale(t1, c1), cscale(t2, c2)));
        dfc b2 = cadd(v[0], cadd(cscale(t1, c2), cscale(t2, c1)));
        dfc r1 = rot90<INV>(cadd(cscale(t3, s1), cscale(t4, s2)));
        dfc r2 = rot90<INV>(csub(cscale(t3, s2), cscale(t4, s1)));
        v[0] = cadd(v[0], cadd(t1, t2));
        v[1] = cadd(b1, r1);
        v[4] = csub(b1, r1);
        v[2] = cadd(b2, r2);
        v[3] = csub(b2, r2);
    }
}

// n / d for a divisor fixed per stage: multiply-high by m = ceil(2^32 / d), exact
// for n < 2^32 / d (every index here is far below that)
struct StageDiv {
    unsigned d, m;
    __device__ __forceinline__ explicit StageDiv(int dv) : d((unsigned)dv), m(dv > 1 ? 0xFFFFFFFFu / (unsigned)dv + 1u : 0u) {}
    __device__ __forceinline__ int div(int n) const { return d == 1 ? n : (int)__umulhi((unsigned)n, m); }
};

template <int R, bool INV, class V>
__device__ __forceinline__ void fft_stage(const V *src, V *dst, int nrows, int stride, int n, int Ns,
                                          const V *__restrict__ tw, int tid, int nthr) {
    const int nb = n / R;
    const int tstep = n / (Ns * R);
    const int total = nrows * nb;
    const StageDiv dnb(nb), dns(Ns);
    for (int idx = tid; idx < total; idx += nthr) {
        int row = dnb.div(idx);
        int j = idx - row * nb;
        const V *x = src + row * stride;
        V *y = dst + row * stride;
        int k = j - dns.div(j) * Ns;
        V v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = x[fpad(j + r * nb)];
        if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) {
                const V w = tw[k * r * tstep];   // global or shared memory
                v[r] = INV ? cmulconj(v[r], w) : cmul(v[r], w);
            }
        }
        dft_small<R, INV>(v);
        int base = (j - k) * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) y[fpad(base + r * Ns)] = v[r];
    }
}

// Transform nrows rows of n complex points held in `a` (row stride `stride`,
// at least frow(n); element i of a row at fpad(i)), using `b` as the
// ping-pong buffer.  Returns the buffer holding the result (same layout).
// All threads of the block must call it; ends with __syncthreads().
template <bool INV, class V>
__device__ V *fft_rows(V *a, V *b, int nrows, int stride, const FftPlan &P, const V *__restrict__ tw, int tid,
                       int nthr) {
    V *src = a, *dst = b;
    int Ns = 1;
    for (int s = 0; s < P.nstage; ++s) {
        int R = P.rad[s];
        switch (R) {
            case 4: fft_stage<4, INV>(src, dst, nrows, stride, P.n, Ns, tw, tid, nthr); break;
            case 2: fft_stage<2, INV>(src, dst, nrows, stride, P.n, Ns, tw, tid, nthr); break;
            case 3: fft_stage<3, INV>(src, dst, nrows, stride, P.n, Ns, tw, tid, nthr); break;
            default: fft_stage<5, INV>(src, dst, nrows, stride, P.n, Ns, tw, tid, nthr); break;
        }
        __syncthreads();
        V *t = src;
        src = dst;
        dst = t;
        Ns *= R;
    }
    return src;
}

}  // namespace aeros
