// Register butterflies shared by the Stockham passes (gw_fft.cuh) and the
// register DFTs of the fused kernels (gw_dft.cuh): DFTs of length 2, 3, 4,
// 5, 8 and 16 on values held by one thread (forward W = exp(-2 pi i / R),
// inverse its conjugate, no scaling).
#pragma once

#include "gw_common.cuh"

template <bool INV>
__host__ __device__ __forceinline__ float2 conj_if(float2 w) {
  if (INV) w.y = -w.y;
  return w;
}

// x * exp(-+ i pi/2): forward multiplies by -i, inverse by +i
template <bool INV>
__host__ __device__ __forceinline__ float2 mul_mi(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// a + mul_mi(e) and a - mul_mi(e) in scalar form: the rotation by -+i is
// folded into the operands (a paired add would need the swapped halves
// made first)
template <bool INV>
__host__ __device__ __forceinline__ float2 add_mi(float2 a, float2 e) {
  return INV ? make_float2(a.x - e.y, a.y + e.x) : make_float2(a.x + e.y, a.y - e.x);
}
template <bool INV>
__host__ __device__ __forceinline__ float2 sub_mi(float2 a, float2 e) {
  return INV ? make_float2(a.x + e.y, a.y - e.x) : make_float2(a.x - e.y, a.y + e.x);
}

template <bool INV>
__host__ __device__ __forceinline__ void dft2(float2 &a0, float2 &a1) {
  const float2 s = cadd(a0, a1), d = csub(a0, a1);
  a0 = s;
  a1 = d;
}

template <bool INV>
__host__ __device__ __forceinline__ void dft4(float2 &a0, float2 &a1, float2 &a2,
                                     float2 &a3) {
  const float2 s0 = cadd(a0, a2), d0 = csub(a0, a2);
  const float2 s1 = cadd(a1, a3), e = csub(a1, a3);
  a0 = cadd(s0, s1);
  a2 = csub(s0, s1);
  a1 = add_mi<INV>(d0, e);
  a3 = sub_mi<INV>(d0, e);
}

// W_16^m (forward sign); m in 0..15
__host__ __device__ __forceinline__ float2 w16(int m) {
  constexpr float c1 = 0.92387953251128674f, s1 = 0.38268343236508978f;
  constexpr float c2 = 0.70710678118654752f;
  switch (m & 15) {
    case 0: return make_float2(1.f, 0.f);
    case 1: return make_float2(c1, -s1);
    case 2: return make_float2(c2, -c2);
    case 3: return make_float2(s1, -c1);
    case 4: return make_float2(0.f, -1.f);
    case 5: return make_float2(-s1, -c1);
    case 6: return make_float2(-c2, -c2);
    case 7: return make_float2(-c1, -s1);
    case 8: return make_float2(-1.f, 0.f);
    case 9: return make_float2(-c1, s1);
    case 10: return make_float2(-c2, c2);
    case 11: return make_float2(-s1, c1);
    case 12: return make_float2(0.f, 1.f);
    case 13: return make_float2(s1, c1);
    case 14: return make_float2(c2, c2);
    default: return make_float2(c1, s1);
  }
}

// In-register R-point DFT.  Output k ends in slot out_slot<R>(k).
template <int R>
__host__ __device__ constexpr int out_slot(int k) {
  return R == 16 ? (k % 4) * 4 + k / 4 : R == 8 ? (k % 4) * 2 + k / 4 : k;
}

// 3-point DFT: y0 = a0+a1+a2, y1,2 = a0 - (a1+a2)/2 -+ i s (a1-a2) with
// s = sin(2 pi/3) (forward; the inverse swaps the sign of i).
template <bool INV>
__host__ __device__ __forceinline__ void dft3(float2 *v) {
  constexpr float s = 0.86602540378443865f;
  const float2 t1 = cadd(v[1], v[2]);
  const float2 t2 = make_float2(v[0].x - 0.5f * t1.x, v[0].y - 0.5f * t1.y);
  const float2 d = csub(v[1], v[2]);
  const float2 sd = make_float2(s * d.x, s * d.y);
  v[0] = cadd(v[0], t1);
  v[1] = add_mi<INV>(t2, sd);
  v[2] = sub_mi<INV>(t2, sd);
}

// 5-point DFT with c_k = cos(2 pi k/5), s_k = sin(2 pi k/5):
// b1 = a0 + c1 (a1+a4) + c2 (a2+a3), b2 = a0 + c2 (a1+a4) + c1 (a2+a3),
// d1 = s1 (a1-a4) + s2 (a2-a3), d2 = s2 (a1-a4) - s1 (a2-a3);
// forward y1 = b1 - i d1, y4 = b1 + i d1, y2 = b2 - i d2, y3 = b2 + i d2.
template <bool INV>
__host__ __device__ __forceinline__ void dft5(float2 *v) {
  constexpr float c1 = 0.30901699437494742f, c2 = -0.80901699437494742f;
  constexpr float s1 = 0.95105651629515357f, s2 = 0.58778525229247313f;
  const float2 t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
  const float2 t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
  const float2 b1 = make_float2(v[0].x + c1 * t1.x + c2 * t2.x, v[0].y + c1 * t1.y + c2 * t2.y);
  const float2 b2 = make_float2(v[0].x + c2 * t1.x + c1 * t2.x, v[0].y + c2 * t1.y + c1 * t2.y);
  const float2 d1 = make_float2(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y);
  const float2 d2 = make_float2(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y);
  // y1 = b1 - i d1 (forward), y4 = b1 + i d1; likewise y2, y3 from b2, d2
  v[0] = cadd(v[0], cadd(t1, t2));
  v[1] = add_mi<INV>(b1, d1);
  v[4] = sub_mi<INV>(b1, d1);
  v[2] = add_mi<INV>(b2, d2);
  v[3] = sub_mi<INV>(b2, d2);
}

template <int R, bool INV>
__host__ __device__ __forceinline__ void dft(float2 *v) {
  if constexpr (R == 2) {
    dft2<INV>(v[0], v[1]);
  } else if constexpr (R == 3) {
    dft3<INV>(v);
  } else if constexpr (R == 5) {
    dft5<INV>(v);
  } else if constexpr (R == 4) {
    dft4<INV>(v[0], v[1], v[2], v[3]);
  } else if constexpr (R == 8) {
    // n = 2 n1 + n2; four-point DFTs over n1, twiddle W8^{n2 k1}, pairs
#pragma unroll
    for (int n2 = 0; n2 < 2; ++n2) dft4<INV>(v[n2], v[n2 + 2], v[n2 + 4], v[n2 + 6]);
#pragma unroll
    for (int k1 = 1; k1 < 4; ++k1) v[1 + 2 * k1] = cmul(v[1 + 2 * k1], conj_if<INV>(w16(2 * k1)));
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) dft2<INV>(v[2 * k1], v[2 * k1 + 1]);
  } else {
    static_assert(R == 16, "radix");
    // n = 4 n1 + n2; four-point DFTs over n1, twiddle W16^{n2 k1}, over n2
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2)
      dft4<INV>(v[n2], v[n2 + 4], v[n2 + 8], v[n2 + 12]);
#pragma unroll
    for (int n2 = 1; n2 < 4; ++n2)
#pragma unroll
      for (int k1 = 1; k1 < 4; ++k1)
        v[n2 + 4 * k1] = cmul(v[n2 + 4 * k1], conj_if<INV>(w16(n2 * k1)));
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1)
      dft4<INV>(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
  }
}

