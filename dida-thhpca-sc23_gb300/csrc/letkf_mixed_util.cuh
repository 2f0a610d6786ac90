// letkf_mixed_util.cuh -- small device helpers shared by the mixed-precision
// core kernels: BF16 hi/lo splitting and cp.async row copies.
#pragma once

// float -> double without the FP64 pipe (which is narrow on this part): the
// conversion is exact, so it is done on the integer pipe from the bits.
// Zeros and subnormal floats become signed zeros; infinities and NaNs keep
// their kind.
__device__ __forceinline__ double lg_f2d_bits(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned sign = u & 0x80000000u, ex = (u >> 23) & 0xffu, man = u & 0x7fffffu;
    unsigned hi, lo;
    if (ex == 0u) {
        hi = sign;
        lo = 0u;
    } else {
        const unsigned e64 = (ex == 0xffu) ? 0x7ffu : ex + 896u;   // 1023 - 127
        hi = sign | (e64 << 20) | (man >> 3);
        lo = man << 29;
    }
    return __hiloint2double((int)hi, (int)lo);
}

#include <cuda_bf16.h>
#include <stdint.h>

// hi/lo BF16 split of two columns m, m + 1 over 8 observations: x[j] holds the
// FP32 pair (column m, column m + 1) of observation j.  Gives the same bits as
// split8 on each column (hi = bf16(v), lo = bf16(v - hi), observation 2i in
// the low half of word i) with the residuals as packed f32x2 differences.
__device__ __forceinline__ void split8x2(const unsigned long long *x, uint4 &hi0, uint4 &lo0, uint4 &hi1,
                                         uint4 &lo1)
{
    uint32_t h0[4], l0[4], h1[4], l1[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        float a0, a1, b0, b1;                       // a: observation 2i, b: 2i + 1
        asm("mov.b64 {%0, %1}, %2;" : "=f"(a0), "=f"(a1) : "l"(x[2 * i]));
        asm("mov.b64 {%0, %1}, %2;" : "=f"(b0), "=f"(b1) : "l"(x[2 * i + 1]));
        __nv_bfloat162 p0 = __floats2bfloat162_rn(a0, b0), p1 = __floats2bfloat162_rn(a1, b1);
        h0[i] = *reinterpret_cast<uint32_t *>(&p0);
        h1[i] = *reinterpret_cast<uint32_t *>(&p1);
        unsigned long long ha, hb, ra, rb;
        asm("mov.b64 %0, {%1, %2};" : "=l"(ha) : "r"(h0[i] << 16), "r"(h1[i] << 16));
        asm("mov.b64 %0, {%1, %2};" : "=l"(hb) : "r"(h0[i] & 0xffff0000u), "r"(h1[i] & 0xffff0000u));
        asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(ra) : "l"(x[2 * i]), "l"(ha));
        asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(rb) : "l"(x[2 * i + 1]), "l"(hb));
        asm("mov.b64 {%0, %1}, %2;" : "=f"(a0), "=f"(a1) : "l"(ra));
        asm("mov.b64 {%0, %1}, %2;" : "=f"(b0), "=f"(b1) : "l"(rb));
        p0 = __floats2bfloat162_rn(a0, b0);
        p1 = __floats2bfloat162_rn(a1, b1);
        l0[i] = *reinterpret_cast<uint32_t *>(&p0);
        l1[i] = *reinterpret_cast<uint32_t *>(&p1);
    }
    hi0 = make_uint4(h0[0], h0[1], h0[2], h0[3]);
    lo0 = make_uint4(l0[0], l0[1], l0[2], l0[3]);
    hi1 = make_uint4(h1[0], h1[1], h1[2], h1[3]);
    lo1 = make_uint4(l1[0], l1[1], l1[2], l1[3]);
}

#include <cuda_fp16.h>

// The A build's operands are split into FP16 hi/lo parts (11 significant
// bits each, so hi + lo keeps about 22 of a float's 24: 2^6 times closer than
// BF16 hi/lo at the same tensor-core rate).  FP16's range is narrow, so the
// operands are first multiplied by a power of two 2^E chosen from the largest
// magnitude m among them (H records it, as float bits, for the whole run):
// m 2^E < 2^15 keeps every hi part at most 32768 < 65504 and puts values down
// to 2^-29 m in FP16's normal range.  Powers of two commute with rounding, so
// the products times 2^-2E are those of the unscaled operands.
// E for the largest magnitude m (bits of a non-negative float): 0 when m is
// zero or not finite, else 15 - e with m < 2^e, clamped to [-60, 60] so that
// 2^E and 2^-2E are normal floats.
__device__ __forceinline__ int lg_f16_scale_exp(unsigned mbits)
{
    const int ex = (int)((mbits >> 23) & 0xffu);
    if (mbits == 0u || ex == 0xff) return 0;
    return min(max(141 - ex, -60), 60);      // normal m < 2^(ex - 126); subnormal m: the clamp
}
__device__ __forceinline__ float lg_pow2f(int e) { return __uint_as_float((unsigned)(e + 127) << 23); }

// hi/lo FP16 split of two columns m, m + 1 over 8 observations, laid out as
// split8x2's BF16 parts: hi = f16(v), lo = f16(v - hi), observation 2i in the
// low half of word i; the residuals as packed f32x2 differences.
__device__ __forceinline__ void split8x2_f16(const unsigned long long *x, uint4 &hi0, uint4 &lo0, uint4 &hi1,
                                             uint4 &lo1)
{
    uint32_t h0[4], l0[4], h1[4], l1[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        float a0, a1, b0, b1;                       // a: observation 2i, b: 2i + 1
        asm("mov.b64 {%0, %1}, %2;" : "=f"(a0), "=f"(a1) : "l"(x[2 * i]));
        asm("mov.b64 {%0, %1}, %2;" : "=f"(b0), "=f"(b1) : "l"(x[2 * i + 1]));
        __half2 p0 = __floats2half2_rn(a0, b0), p1 = __floats2half2_rn(a1, b1);
        h0[i] = *reinterpret_cast<uint32_t *>(&p0);
        h1[i] = *reinterpret_cast<uint32_t *>(&p1);
        const float2 f0 = __half22float2(p0), f1 = __half22float2(p1);
        unsigned long long ha, hb, ra, rb;
        asm("mov.b64 %0, {%1, %2};" : "=l"(ha) : "f"(f0.x), "f"(f1.x));
        asm("mov.b64 %0, {%1, %2};" : "=l"(hb) : "f"(f0.y), "f"(f1.y));
        asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(ra) : "l"(x[2 * i]), "l"(ha));
        asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(rb) : "l"(x[2 * i + 1]), "l"(hb));
        asm("mov.b64 {%0, %1}, %2;" : "=f"(a0), "=f"(a1) : "l"(ra));
        asm("mov.b64 {%0, %1}, %2;" : "=f"(b0), "=f"(b1) : "l"(rb));
        p0 = __floats2half2_rn(a0, b0);
        p1 = __floats2half2_rn(a1, b1);
        l0[i] = *reinterpret_cast<uint32_t *>(&p0);
        l1[i] = *reinterpret_cast<uint32_t *>(&p1);
    }
    hi0 = make_uint4(h0[0], h0[1], h0[2], h0[3]);
    lo0 = make_uint4(l0[0], l0[1], l0[2], l0[3]);
    hi1 = make_uint4(h1[0], h1[1], h1[2], h1[3]);
    lo1 = make_uint4(l1[0], l1[1], l1[2], l1[3]);
}

// hi/lo FP16 split of 8 floats into two 16-byte chunks.
__device__ __forceinline__ void split8_f16(const float *v, uint4 &hi, uint4 &lo)
{
    uint32_t h[4], l[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        __half2 hh = __floats2half2_rn(v[2 * j], v[2 * j + 1]);
        const float2 f = __half22float2(hh);
        __half2 ll = __floats2half2_rn(v[2 * j] - f.x, v[2 * j + 1] - f.y);
        h[j] = *reinterpret_cast<uint32_t *>(&hh);
        l[j] = *reinterpret_cast<uint32_t *>(&ll);
    }
    hi = make_uint4(h[0], h[1], h[2], h[3]);
    lo = make_uint4(l[0], l[1], l[2], l[3]);
}

// 16-byte global -> shared copies that bypass the registers (cp.async, L2 only).
__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

__device__ __forceinline__ uint32_t pack_bf16(float a, float b)
{
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t *>(&h);
}

// hi/lo BF16 split of 8 floats into two 16-byte chunks.
__device__ __forceinline__ void split8(const float *v, uint4 &hi, uint4 &lo)
{
    uint32_t h[4], l[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const __nv_bfloat16 h0 = __float2bfloat16_rn(v[2 * j]), h1 = __float2bfloat16_rn(v[2 * j + 1]);
        const float r0 = v[2 * j] - __bfloat162float(h0), r1 = v[2 * j + 1] - __bfloat162float(h1);
        __nv_bfloat162 hh;
        hh.x = h0;
        hh.y = h1;
        h[j] = *reinterpret_cast<uint32_t *>(&hh);
        l[j] = pack_bf16(r0, r1);
    }
    hi = make_uint4(h[0], h[1], h[2], h[3]);
    lo = make_uint4(l[0], l[1], l[2], l[3]);
}

