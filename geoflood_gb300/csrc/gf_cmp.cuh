/*
 * FP64 comparisons and min / max on the integer pipe.
 *
 * On this GPU an FP64 warp instruction occupies the FP64 pipe for tens of
 * cycles while an integer instruction issues in two; comparisons and
 * min / max of doubles are a quarter of the patch update's FP64-pipe
 * instructions. With FAST = true these helpers compare the IEEE bit
 * patterns instead:
 *   - against zero they are exact (x > 0, x < 0, x == 0 with either zero);
 *   - between two values they use the order-preserving integer key of the
 *     bit pattern, which agrees with IEEE ordering except that -0 sorts
 *     below +0 (IEEE: equal). Inputs are never NaN here.
 * With FAST = false they are the IEEE operations themselves, so the
 * contraction-free build keeps the reference's arithmetic bit for bit.
 */
#ifndef GF_CMP_CUH
#define GF_CMP_CUH

__device__ __forceinline__ long long gf_bits(double x) { return __double_as_longlong(x); }

/* order-preserving signed key: larger double <=> larger key */
__device__ __forceinline__ long long gf_okey(double x)
{
    const long long b = __double_as_longlong(x);
    return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}

template <bool F> __device__ __forceinline__ bool d_lt(double a, double b)
{
    if (F) return gf_okey(a) < gf_okey(b);
    return a < b;
}
template <bool F> __device__ __forceinline__ bool d_le(double a, double b)
{
    if (F) return gf_okey(a) <= gf_okey(b);
    return a <= b;
}
template <bool F> __device__ __forceinline__ bool d_gt(double a, double b) { return d_lt<F>(b, a); }
template <bool F> __device__ __forceinline__ bool d_ge(double a, double b) { return d_le<F>(b, a); }

/* against zero: exact for both zeros */
template <bool F> __device__ __forceinline__ bool d_gtz(double x)
{
    if (F) return gf_bits(x) > 0;
    return x > 0.0;
}
template <bool F> __device__ __forceinline__ bool d_ltz(double x)
{
    if (F) {
        const long long b = gf_bits(x);
        return b < 0 && (b << 1) != 0;
    }
    return x < 0.0;
}
template <bool F> __device__ __forceinline__ bool d_lez(double x) { return !d_gtz<F>(x); }
template <bool F> __device__ __forceinline__ bool d_gez(double x) { return !d_ltz<F>(x); }
template <bool F> __device__ __forceinline__ bool d_eqz(double x)
{
    if (F) return (gf_bits(x) << 1) == 0;
    return x == 0.0;
}

template <bool F> __device__ __forceinline__ double d_max(double a, double b)
{
    if (F) return gf_okey(a) < gf_okey(b) ? b : a;
    return fmax(a, b);
}
template <bool F> __device__ __forceinline__ double d_min(double a, double b)
{
    if (F) return gf_okey(b) < gf_okey(a) ? b : a;
    return fmin(a, b);
}
/* both operands >= +0 (or -0): the raw bit patterns order correctly */
template <bool F> __device__ __forceinline__ double d_max_nn(double a, double b)
{
    if (F) return gf_bits(a) < gf_bits(b) ? b : a;
    return fmax(a, b);
}

/* 1/y from the hardware's approximate FP64 reciprocal refined by two
 * Newton-Raphson steps r <- r + r (1 - y r) (quadratic convergence: about
 * 2^-84 relative before the last rounding, i.e. within an ulp of the
 * correctly rounded quotient). For normal, non-zero y only: the inputs
 * here are depths, speeds and their differences away from zero. */
__device__ __forceinline__ double gf_rcp(double y)
{
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(y));
    double e = fma(-y, r, 1.0);
    r = fma(r, e, r);
    e = fma(-y, r, 1.0);
    return fma(r, e, r);
}

/* x / y: the IEEE quotient, or x * gf_rcp(y) in the production build */
template <bool F> __device__ __forceinline__ double d_div(double x, double y)
{
    if (F) return x * gf_rcp(y);
    return x / y;
}

#endif
