/*
 * nr_math.h — arithmetic shared, bit for bit, by the CUDA kernels and host code.
 *
 *  - PCG32 (XSH-RR 64/32), seeded the way NRAPS's src/rand.rs:49-71 seeds it
 *    (state 0, inc = stream<<1|1, step, state += seed, step; i.e. the
 *    pcg32_srandom_r procedure of pcg-c-basic), with the wall-clock seed
 *    replaced by an explicit one; output step as src/rand.rs:73-85.
 *  - Uniform draws: the f32 draw of src/rand.rs:94-100, (u as f32) * 2^-32
 *    (the literal 2.3283064E-10 rounds to exactly 2^-32 in f32), which can
 *    return 1.0; its FP64 counterpart u * 2^-32.
 *  - nr_log / nr_logf: the natural logarithm both sides evaluate.  Method:
 *    Cody & Waite reduction x = 2^e * m with m in [sqrt(1/2), sqrt(2)), then
 *    ln m = 2 atanh(s), s = (m-1)/(m+1), summed as the Taylor series
 *    2s(1 + s^2/3 + s^4/5 + ...) (Abramowitz & Stegun 4.1.27), and
 *    ln x = e*ln2_hi + (e*ln2_lo + ln m) with ln 2 split into a 32-bit head
 *    (16-bit for f32) so that e*ln2_hi is exact.  Only correctly rounded IEEE
 *    operations are used (+, -, *, /, fma) and on the device they are the
 *    explicit round-to-nearest intrinsics, which the compiler never contracts,
 *    so CPU and GPU return identical bits.  Host code that includes this must
 *    be compiled with -ffp-contract=off.
 *  - Fixed-point scores: a k-estimator score v >= 0 is rounded once to an
 *    integer multiple of 2^-32 and summed in uint64; the sum is exact, so k is
 *    independent of the order in which threads add their scores.
 */
#ifndef NR_MATH_H
#define NR_MATH_H

#include <stdint.h>

#include <cmath>
#include <cstring>
#if defined(__CUDACC__)
#define NR_HD __host__ __device__ __forceinline__
#else
#define NR_HD inline
#endif

/* ---- IEEE primitives that never contract ------------------------------- */
#if defined(__CUDA_ARCH__)
#define NR_ADD(a, b)    __dadd_rn((a), (b))
#define NR_MUL(a, b)    __dmul_rn((a), (b))
#define NR_DIV(a, b)    __ddiv_rn((a), (b))
#define NR_FMA(a, b, c) __fma_rn((a), (b), (c))
#define NR_ADDF(a, b)   __fadd_rn((a), (b))
#define NR_MULF(a, b)   __fmul_rn((a), (b))
#define NR_DIVF(a, b)   __fdiv_rn((a), (b))
#define NR_FMAF(a, b, c) __fmaf_rn((a), (b), (c))
#else
#define NR_ADD(a, b)    ((a) + (b))
#define NR_MUL(a, b)    ((a) * (b))
#define NR_DIV(a, b)    ((a) / (b))
#define NR_FMA(a, b, c) std::fma((a), (b), (c))
#define NR_ADDF(a, b)   ((a) + (b))
#define NR_MULF(a, b)   ((a) * (b))
#define NR_DIVF(a, b)   ((a) / (b))
#define NR_FMAF(a, b, c) std::fmaf((a), (b), (c))
#endif

NR_HD uint64_t nr_bits64(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b; std::memcpy(&b, &x, 8); return b;
#endif
}
NR_HD double nr_from_bits64(uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double x; std::memcpy(&x, &b, 8); return x;
#endif
}
NR_HD uint32_t nr_bits32(float x) {
#if defined(__CUDA_ARCH__)
    return (uint32_t)__float_as_uint(x);
#else
    uint32_t b; std::memcpy(&b, &x, 4); return b;
#endif
}
NR_HD float nr_from_bits32(uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(b);
#else
    float x; std::memcpy(&x, &b, 4); return x;
#endif
}

/* ---- PCG32 ---------------------------------------------------------------- */
#define NR_PCG_MULT 6364136223846793005ULL

typedef struct nr_pcg32 { uint64_t state, inc; } nr_pcg32;

NR_HD uint32_t nr_pcg32_next(nr_pcg32* r) {
    uint64_t old = r->state;
    r->state = old * NR_PCG_MULT + r->inc;
    uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
    uint32_t rot = (uint32_t)(old >> 59);
#if defined(__CUDA_ARCH__)
    return __funnelshift_r(xs, xs, rot);
#else
    return (xs >> rot) | (xs << ((0u - rot) & 31u));
#endif
}

/* stream = history id, seed = generation seed.  The first step from state 0
   lands on state == inc, so the two-step seeding folds to one multiply-add
   before the second step. */
NR_HD nr_pcg32 nr_pcg32_seeded(uint64_t seed, uint64_t stream) {
    nr_pcg32 r;
    r.inc = (stream << 1) | 1ULL;
    r.state = r.inc + seed;            /* state after step 1 is inc; += seed */
    nr_pcg32_next(&r);                 /* step 2                              */
    return r;
}

/* SplitMix64 finaliser (Steele, Lea & Flood, OOPSLA 2014). */
NR_HD uint64_t nr_splitmix64(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

/* Seed of every history stream in generation `gen` of a run seeded `base`. */
NR_HD uint64_t nr_generation_seed(uint64_t base, uint64_t gen) {
    return nr_splitmix64(base ^ nr_splitmix64(gen));
}

/* Reference draws in [0,1] (f32, per rand.rs) and [0,1) (f64). */
NR_HD float nr_u01f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(__uint2float_rn(u), 0x1p-32f);
#else
    return (float)u * 0x1p-32f;
#endif
}
NR_HD double nr_u01d(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __dmul_rn(__uint2double_rn(u), 0x1p-32);
#else
    return (double)u * 0x1p-32;
#endif
}
/* Strictly positive draws in (0,1] for flight lengths, so -ln never is +inf. */
NR_HD float nr_upos_f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(__uint2float_rn((u >> 8) + 1u), 0x1p-24f);
#else
    return (float)((u >> 8) + 1u) * 0x1p-24f;
#endif
}
NR_HD double nr_upos_d(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __dmul_rn(__dadd_rn(__uint2double_rn(u), 1.0), 0x1p-32);
#else
    return ((double)u + 1.0) * 0x1p-32;
#endif
}

/* ---- natural logarithm ---------------------------------------------------- */
NR_HD double nr_log(double x) {
    if (!(x > 0.0)) {
        if (x == 0.0) return nr_from_bits64(0xFFF0000000000000ULL);  /* -inf */
        return nr_from_bits64(0x7FF8000000000000ULL);             /* NaN, x<0  */
    }
    uint64_t b = nr_bits64(x);
    if (b >= 0x7FF0000000000000ULL) return x;                      /* +inf      */
    int e = (int)(b >> 52);
    if (e == 0) {                                                  /* subnormal */
        x = NR_MUL(x, 0x1p54);
        b = nr_bits64(x);
        e = (int)(b >> 52) - 54;
    }
    e -= 1023;
    uint64_t mant = b & 0x000FFFFFFFFFFFFFULL;
    /* m in [1,2); fold m >= sqrt(2) into [sqrt(1/2), 1) */
    if (mant >= 0x6A09E667F3BCDULL) { mant |= 0x3FE0000000000000ULL; e += 1; }
    else                            { mant |= 0x3FF0000000000000ULL; }
    double m = nr_from_bits64(mant);
    double f = NR_ADD(m, -1.0);                                    /* exact     */
    double s = NR_DIV(f, NR_ADD(f, 2.0));
    double z = NR_MUL(s, s);
    double p = 0x1.8618618618618p-5;                               /* 1/21      */
    p = NR_FMA(p, z, 0x1.af286bca1af28p-5);                        /* 1/19      */
    p = NR_FMA(p, z, 0x1.e1e1e1e1e1e1ep-5);                        /* 1/17      */
    p = NR_FMA(p, z, 0x1.1111111111111p-4);                        /* 1/15      */
    p = NR_FMA(p, z, 0x1.3b13b13b13b14p-4);                        /* 1/13      */
    p = NR_FMA(p, z, 0x1.745d1745d1746p-4);                        /* 1/11      */
    p = NR_FMA(p, z, 0x1.c71c71c71c71cp-4);                        /* 1/9       */
    p = NR_FMA(p, z, 0x1.2492492492492p-3);                        /* 1/7       */
    p = NR_FMA(p, z, 0x1.999999999999ap-3);                        /* 1/5       */
    p = NR_FMA(p, z, 0x1.5555555555555p-2);                        /* 1/3       */
    double r = NR_ADD(s, s);                                       /* 2s        */
    double lm = NR_FMA(r, NR_MUL(z, p), r);                        /* 2s(1+zp)  */
    double de = (double)e;
    return NR_FMA(de, 0x1.62e42ff000000p-1, NR_FMA(de, -0x1.718432a1b0e26p-35, lm));
}

NR_HD float nr_logf(float x) {
    if (!(x > 0.0f)) {
        if (x == 0.0f) return nr_from_bits32(0xFF800000u);         /* -inf      */
        return nr_from_bits32(0x7FC00000u);                        /* NaN       */
    }
    uint32_t b = nr_bits32(x);
    if (b >= 0x7F800000u) return x;
    int e = (int)(b >> 23);
    if (e == 0) {
        x = NR_MULF(x, 0x1p25f);
        b = nr_bits32(x);
        e = (int)(b >> 23) - 25;
    }
    e -= 127;
    uint32_t mant = b & 0x007FFFFFu;
    if (mant >= 0x3504F3u) { mant |= 0x3F000000u; e += 1; }       /* m >= sqrt2 */
    else                   { mant |= 0x3F800000u; }
    float m = nr_from_bits32(mant);
    float f = NR_ADDF(m, -1.0f);
    float s = NR_DIVF(f, NR_ADDF(f, 2.0f));
    float z = NR_MULF(s, s);
    float p = 0x1.c71c72p-4f;                                      /* 1/9       */
    p = NR_FMAF(p, z, 0x1.24924ap-3f);                             /* 1/7       */
    p = NR_FMAF(p, z, 0x1.99999ap-3f);                             /* 1/5       */
    p = NR_FMAF(p, z, 0x1.555556p-2f);                             /* 1/3       */
    float r = NR_ADDF(s, s);
    float lm = NR_FMAF(r, NR_MULF(z, p), r);
    float de = (float)e;
    return NR_FMAF(de, 0x1.62e4p-1f, NR_FMAF(de, 0x1.7f7d1cp-20f, lm));
}

/* ---- fixed-point k scores -------------------------------------------------- */
#define NR_FIX_SCALE 0x1p32
NR_HD uint64_t nr_fix(double v) {
    if (!(v > 0.0)) return 0;                     /* 0, negatives, NaN        */
    if (v >= 0x1p31) return 0x7FFFFFFFFFFFFFFFULL; /* saturate (never in range) */
#if defined(__CUDA_ARCH__)
    return __double2ull_rn(__dmul_rn(v, NR_FIX_SCALE));
#else
    return (uint64_t)std::nearbyint(v * NR_FIX_SCALE);
#endif
}
NR_HD double nr_unfix(uint64_t q) { return (double)q * 0x1p-32; }

#endif /* NR_MATH_H */
