// Device comparators: one distance computed cooperatively by a group of G
// lanes (G a power of two <= 32) that stream the row in 16-byte chunks.
//
// Each metric restates the reference comparator's arithmetic
// (lib/NGT/PrimitiveComparatorX86.h:100-1190, lib/NGT/PrimitiveComparatorNoArch.h:30-390):
//   * element-wise sums in float lanes (integer lanes for uint8 / bit metrics,
//     which are therefore exact), then the reference's final formula;
//   * the float result equals the reference's (float)f(double) result whenever
//     the lane sums agree (always for integer data: float(sqrt((double)s)) is the
//     correctly rounded sqrtf(s) for any float s, since 53 >= 2*24+2).
#pragma once
#include <cuda_fp16.h>
#include <cstdint>
#include "ngt_types.h"

namespace ngtg {

template <ObjType OT> struct ObjTraits;
template <> struct ObjTraits<ObjType::Float> { typedef float T; static constexpr int kPerChunk = 4; };
template <> struct ObjTraits<ObjType::Float16> { typedef __half T; static constexpr int kPerChunk = 8; };
template <> struct ObjTraits<ObjType::Uint8> { typedef uint8_t T; static constexpr int kPerChunk = 16; };
template <> struct ObjTraits<ObjType::Bfloat16> { typedef uint16_t T; static constexpr int kPerChunk = 8; };
template <> struct ObjTraits<ObjType::Qsint8> { typedef int8_t T; static constexpr int kPerChunk = 16; };

template <ObjType OT>
__device__ __forceinline__ void unpack(const uint4& v, float* f);
template <>
__device__ __forceinline__ void unpack<ObjType::Float>(const uint4& v, float* f) {
  f[0] = __uint_as_float(v.x); f[1] = __uint_as_float(v.y);
  f[2] = __uint_as_float(v.z); f[3] = __uint_as_float(v.w);
}
template <>
__device__ __forceinline__ void unpack<ObjType::Float16>(const uint4& v, float* f) {
  const __half2* h = reinterpret_cast<const __half2*>(&v);
#pragma unroll
  for (int i = 0; i < 4; i++) {
    float2 t = __half22float2(h[i]);
    f[2 * i] = t.x; f[2 * i + 1] = t.y;
  }
}
template <>
__device__ __forceinline__ void unpack<ObjType::Bfloat16>(const uint4& v, float* f) {
  const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
  for (int i = 0; i < 4; i++) {
    f[2 * i] = __uint_as_float(w[i] << 16);
    f[2 * i + 1] = __uint_as_float(w[i] & 0xffff0000u);
  }
}
template <>
__device__ __forceinline__ void unpack<ObjType::Qsint8>(const uint4& v, float* f) {
  const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
  for (int i = 0; i < 16; i++) f[i] = (float)(int8_t)((w[i >> 2] >> ((i & 3) * 8)) & 0xffu);
}
template <>
__device__ __forceinline__ void unpack<ObjType::Uint8>(const uint4& v, float* f) {
  const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
  for (int i = 0; i < 16; i++) f[i] = (float)((w[i >> 2] >> ((i & 3) * 8)) & 0xffu);
}

// Metric accumulator.  add() consumes one 16-byte chunk of the query and of
// the row; chunk_index is the chunk's position in the row (Lorentz needs to
// know which element is the first one).
template <ObjType OT, Metric M>
struct Acc {
  float f0 = 0.f, f1 = 0.f, f2 = 0.f;
  uint32_t i0 = 0, i1 = 0;

  __device__ __forceinline__ void add(const uint4& q, const uint4& x, int chunk_index) {
    if constexpr (OT == ObjType::Uint8 && (M == Metric::L2 || M == Metric::InnerProduct || M == Metric::Quint8L2)) {
      const uint32_t qa[4] = {q.x, q.y, q.z, q.w}, xa[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
      for (int i = 0; i < 4; i++) {
        // (a-b)^2 = a^2 + b^2 - 2ab, all in exact unsigned 32-bit arithmetic.
        i0 += __dp4a(qa[i], qa[i], 0u) + __dp4a(xa[i], xa[i], 0u);
        i1 += __dp4a(qa[i], xa[i], 0u);
      }
    } else if constexpr (OT == ObjType::Qsint8 && M == Metric::L2) {
      const int qa[4] = {(int)q.x, (int)q.y, (int)q.z, (int)q.w}, xa[4] = {(int)x.x, (int)x.y, (int)x.z, (int)x.w};
#pragma unroll
      for (int i = 0; i < 4; i++) {
        // (a-b)^2 = a^2 + b^2 - 2ab over signed bytes, exact 32-bit arithmetic
        i0 += (uint32_t)(__dp4a(qa[i], qa[i], 0) + __dp4a(xa[i], xa[i], 0));
        i1 += (uint32_t)__dp4a(qa[i], xa[i], 0);
      }
    } else if constexpr (OT == ObjType::Qsint8 && (M == Metric::InnerProduct || M == Metric::NormalizedCosine)) {
      // signed query codes . unsigned stored codes (the codes shifted by 127), exact;
      // i0 counts the elements (the padded dimension the reference's constant uses)
      const uint32_t qa[4] = {q.x, q.y, q.z, q.w}, xa[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
      for (int i = 0; i < 4; i++) {
        int r;
        asm("dp4a.s32.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(qa[i]), "r"(xa[i]), "r"(0));
        i1 += (uint32_t)r;
      }
      i0 += 16u;
    } else if constexpr (OT == ObjType::Uint8 && M == Metric::L1) {
      i0 += __vsadu4(q.x, x.x) + __vsadu4(q.y, x.y) + __vsadu4(q.z, x.z) + __vsadu4(q.w, x.w);
    } else if constexpr (M == Metric::Hamming) {
      i0 += __popc(q.x ^ x.x) + __popc(q.y ^ x.y) + __popc(q.z ^ x.z) + __popc(q.w ^ x.w);
    } else if constexpr (M == Metric::Jaccard) {
      i0 += __popc(q.x & x.x) + __popc(q.y & x.y) + __popc(q.z & x.z) + __popc(q.w & x.w);
      i1 += __popc(q.x | x.x) + __popc(q.y | x.y) + __popc(q.z | x.z) + __popc(q.w | x.w);
    } else {
      constexpr int P = ObjTraits<OT>::kPerChunk;
      float a[P], b[P];
      unpack<OT>(q, a);
      unpack<OT>(x, b);
#pragma unroll
      for (int i = 0; i < P; i++) {
        if constexpr (M == Metric::L2 || M == Metric::InnerProduct) {
          float d = a[i] - b[i];
          f0 = __fmaf_rn(d, d, f0);
        } else if constexpr (M == Metric::L1) {
          f0 += fabsf(a[i] - b[i]);
        } else if constexpr (M == Metric::NormalizedCosine || M == Metric::NormalizedAngle ||
                             M == Metric::NormalizedL2) {
          f0 = __fmaf_rn(a[i], b[i], f0);
        } else if constexpr (M == Metric::Cosine || M == Metric::Angle) {
          f0 = __fmaf_rn(a[i], b[i], f0);
          f1 = __fmaf_rn(a[i], a[i], f1);
          f2 = __fmaf_rn(b[i], b[i], f2);
        } else if constexpr (M == Metric::Poincare) {
          float d = a[i] - b[i];
          f0 = __fmaf_rn(d, d, f0);
          f1 = __fmaf_rn(a[i], a[i], f1);
          f2 = __fmaf_rn(b[i], b[i], f2);
        } else if constexpr (M == Metric::Lorentz) {
          // compensated (float-float) sum of the exact products: the reference sums
          // them in double, and acosh near 1 magnifies the error of a plain float sum
          float p = a[i] * b[i];
          float pe = __fmaf_rn(a[i], b[i], -p);
          if (!(chunk_index == 0 && i == 0)) { p = -p; pe = -pe; }
          two_sum_acc(f0, f1, p);
          f1 += pe;
        }
      }
    }
  }

  // Which accumulators a metric uses (only those are reduced across lanes).
  static constexpr bool kUint8Sq =
      (OT == ObjType::Uint8 && (M == Metric::L2 || M == Metric::InnerProduct || M == Metric::Quint8L2)) ||
      (OT == ObjType::Qsint8 && M == Metric::L2);
  static constexpr bool kQsDot = OT == ObjType::Qsint8 && (M == Metric::InnerProduct || M == Metric::NormalizedCosine);
  static constexpr bool kUseI0 = kUint8Sq || kQsDot || (OT == ObjType::Uint8 && M == Metric::L1) ||
                                 M == Metric::Hamming || M == Metric::Jaccard;
  static constexpr bool kUseI1 = kUint8Sq || kQsDot || M == Metric::Jaccard;
  static constexpr bool kUseF0 = !kUseI0;
  static constexpr bool kUseF12 = !kUseI0 && (M == Metric::Cosine || M == Metric::Angle || M == Metric::Poincare);

  // hi += x with the rounding error of the addition carried into lo (Knuth's TwoSum)
  static __device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
    float s = hi + x;
    float bb = s - hi;
    float err = (hi - (s - bb)) + (x - bb);
    hi = s;
    lo += err;
  }

  __device__ __forceinline__ void reduce(int width) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      if (off < width) {
        if constexpr (M == Metric::Lorentz) {
          float h = __shfl_xor_sync(0xffffffffu, f0, off), l = __shfl_xor_sync(0xffffffffu, f1, off);
          // TwoSum's error term is exact whatever the operand order, and f1 + l is
          // commutative, so both lanes of a pair end with the same (hi, lo)
          float lo = f1 + l;
          two_sum_acc(f0, lo, h);
          f1 = lo;
          continue;
        }
        if constexpr (kUseF0) f0 += __shfl_xor_sync(0xffffffffu, f0, off);
        if constexpr (kUseF12) {
          f1 += __shfl_xor_sync(0xffffffffu, f1, off);
          f2 += __shfl_xor_sync(0xffffffffu, f2, off);
        }
        if constexpr (kUseI0) i0 += __shfl_xor_sync(0xffffffffu, i0, off);
        if constexpr (kUseI1) i1 += __shfl_xor_sync(0xffffffffu, i1, off);
      }
    }
  }

  __device__ __forceinline__ float finish() const {
    if constexpr (OT == ObjType::Qsint8 && M == Metric::L2) {
      // the squared sum itself: PrimitiveComparator::compareL2(qsint8) of the x86
      // build (lib/NGT/PrimitiveComparatorX86.h:341-431) takes no square root
      return (float)(int)(i0 - 2u * i1);
    } else if constexpr (kQsDot) {
      // 127*127*n (inner product) or 127*255*n (normalized cosine) minus the dot product,
      // n the padded dimension (PrimitiveComparator::InnerProductQsint8,
      // NormalizedCosineSimilarityQsint8, lib/NGT/PrimitiveComparator.h:376-404)
      const long long c = (M == Metric::InnerProduct ? 127ll * 127ll : 127ll * 255ll) * (long long)i0;
      return (float)(c - (long long)(int)i1);
    } else if constexpr (OT == ObjType::Uint8 && M == Metric::Quint8L2) {
      return (float)(i0 - 2u * i1);    // the squared sum (the reference's quint8 L2 takes no root)
    } else if constexpr (OT == ObjType::Uint8 && (M == Metric::L2 || M == Metric::InnerProduct)) {
      return sqrtf((float)(i0 - 2u * i1));
    } else if constexpr (OT == ObjType::Uint8 && M == Metric::L1) {
      return (float)i0;
    } else if constexpr (M == Metric::Hamming) {
      return (float)i0;
    } else if constexpr (M == Metric::Jaccard) {
      // 1 - |a&b|/|a|b|, evaluated once in double as the reference does.
      return (float)(1.0 - (double)i0 / (double)i1);
    } else if constexpr (M == Metric::L2 || M == Metric::InnerProduct) {
      return sqrtf(f0);
    } else if constexpr (M == Metric::L1) {
      return f0;
    } else if constexpr (M == Metric::NormalizedCosine) {
      float v = 1.0f - f0;
      return v < 0.f ? -v : v;
    } else if constexpr (M == Metric::NormalizedL2) {
      float v = 2.0f - 2.0f * f0;
      return v < 0.f ? 0.f : sqrtf(v);
    } else if constexpr (M == Metric::NormalizedAngle) {
      float c = f0;
      return c >= 1.f ? 0.f : (c <= -1.f ? acosf(-1.f) : acosf(c));
    } else if constexpr (M == Metric::Cosine) {
      float c = f0 / sqrtf(f1 * f2);
      float v = 1.0f - c;
      return v < 0.f ? -v : v;
    } else if constexpr (M == Metric::Angle) {
      float c = f0 / sqrtf(f1 * f2);
      return c >= 1.f ? 0.f : (c <= -1.f ? acosf(-1.f) : acosf(c));
    } else if constexpr (M == Metric::Poincare) {
      // acosh(1 + x) = log1p(x + sqrt(x (x + 2))): keeps the precision of small x,
      // which 1 + x in float would round away (the reference evaluates it in double)
      float x = 2.f * f0 / (1.f - f1) / (1.f - f2);
      return log1pf(x + sqrtf(x * (x + 2.f)));
    } else if constexpr (M == Metric::Lorentz) {
      // s - 1 from the float-float sum (s >= 1 on the hyperboloid), then acosh as above
      float e = (f0 - 1.f) + f1;
      if (!(e >= 0.f)) return e != e ? e : 0.f;
      return log1pf(e + sqrtf(e * (e + 2.f)));
    } else {
      return 0.f;
    }
  }
};

// Distance between the query (16-byte aligned, in shared memory) and row `x`
// (16-byte aligned, global), computed by a group of `width` lanes; `lane` is
// the lane's index inside the group.  Every lane of the group returns the value.
template <ObjType OT, Metric M>
__device__ __forceinline__ float group_distance(const uint4* __restrict__ q, const uint4* __restrict__ x,
                                                int nchunks, int lane, int width) {
  Acc<OT, M> acc;
  for (int c = lane; c < nchunks; c += width) {
    uint4 xv = __ldg(x + c);
    uint4 qv = q[c];
    acc.add(qv, xv, c);
  }
  acc.reduce(width);
  return acc.finish();
}

// Monotone map of a float to unsigned bits (negative distances occur: the
// scalar-quantized inner product), -0 folded to +0; +inf maps to 0xff800000.
__device__ __forceinline__ uint32_t order_bits(float d) {
  const uint32_t b = __float_as_uint(d == 0.0f ? 0.0f : d);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float order_float(uint32_t o) {
  return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}

// Orderable 64-bit key for (distance, id).
__device__ __forceinline__ unsigned long long pack_key(float d, uint32_t id) {
  return ((unsigned long long)order_bits(d) << 32) | id;
}
__device__ __forceinline__ float key_dist(unsigned long long k) { return order_float((uint32_t)(k >> 32)); }

// The comparator of the DVP tree: the search comparator, except for scalar-quantized
// inner-product and normalized-cosine indexes (ObjectSpaceRepository.h:727-745: the
// squared L2 over unsigned bytes, the query's signed codes read as unsigned).
template <ObjType OT, Metric M>
struct TreeSpace {
  static constexpr bool kQuint8 = OT == ObjType::Qsint8 && (M == Metric::InnerProduct || M == Metric::NormalizedCosine);
  static constexpr ObjType ot = kQuint8 ? ObjType::Uint8 : OT;
  static constexpr Metric m = kQuint8 ? Metric::Quint8L2 : M;
};
__device__ __forceinline__ uint32_t key_id(unsigned long long k) { return (uint32_t)k; }

}  // namespace ngtg
