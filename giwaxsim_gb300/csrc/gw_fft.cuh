// Batched power-of-two complex FFTs in shared memory (Stockham autosort).
//
// NB sequences of length M sit back to back in shared memory (buf[f*M+n]).
// Each pass reads every butterfly's R inputs into registers, synchronises,
// then writes the R outputs in Stockham order, so a single buffer suffices.
// Passes are radix-4 with one radix-2 pass when log2(M) is odd.  Twiddles
// come from a shared table tw[t] = exp(-2*pi*i*t/M) made in float64 on the
// host, so no pass evaluates a transcendental.
//
// Sizes and launch shapes: FftShape<M> gives NB (sequences per block) and
// NT (threads) so that every radix-4 pass is 4 butterflies per thread.
#pragma once

#include "gw_common.cuh"

template <int M>
struct FftShape;
template <> struct FftShape<64>   { static constexpr int NB = 16, NT = 64; };
template <> struct FftShape<128>  { static constexpr int NB = 16, NT = 128; };
template <> struct FftShape<256>  { static constexpr int NB = 8,  NT = 128; };
template <> struct FftShape<512>  { static constexpr int NB = 8,  NT = 256; };
template <> struct FftShape<1024> { static constexpr int NB = 4,  NT = 256; };
template <> struct FftShape<2048> { static constexpr int NB = 4,  NT = 512; };
template <> struct FftShape<4096> { static constexpr int NB = 2,  NT = 512; };
template <> struct FftShape<8192> { static constexpr int NB = 1,  NT = 512; };

__host__ __device__ constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n / 2); }

template <bool INV>
__device__ __forceinline__ float2 twid(const float2 *tw, int t) {
  float2 w = tw[t];
  if (INV) w.y = -w.y;
  return w;
}

// In-place radix-4 DFT of (a0,a1,a2,a3); forward uses exp(-i), inverse exp(+i).
template <bool INV>
__device__ __forceinline__ void dft4(float2 &a0, float2 &a1, float2 &a2,
                                     float2 &a3) {
  float2 s0 = cadd(a0, a2), d0 = csub(a0, a2);
  float2 s1 = cadd(a1, a3), d1 = csub(a1, a3);
  // d1 * (-i) forward, d1 * (+i) inverse
  float2 r = INV ? make_float2(-d1.y, d1.x) : make_float2(d1.y, -d1.x);
  a0 = cadd(s0, s1);
  a2 = csub(s0, s1);
  a1 = cadd(d0, r);
  a3 = csub(d0, r);
}

// All threads of the block must call this.  buf: NB*M complex values.
template <int M, int NB, int NT, bool INV>
__device__ __forceinline__ void fft_block(float2 *buf, const float2 *tw) {
  constexpr int LOG2M = ilog2(M);
  constexpr int Q = M / 4;
  constexpr int BF = NB * Q;
  constexpr int PER = BF / NT;
  static_assert(BF % NT == 0, "radix-4 butterflies must split evenly");
  const int tid = threadIdx.x;
  int Ns = 1;
#pragma unroll 1
  for (int pass = 0; pass < LOG2M / 2; ++pass) {
    float2 v[PER][4];
    const int tstride = M / (4 * Ns);
#pragma unroll
    for (int e = 0; e < PER; ++e) {
      const int b = tid + e * NT;
      const int f = b / Q, j = b % Q;
      const float2 *src = buf + f * M;
      float2 a0 = src[j], a1 = src[j + Q], a2 = src[j + 2 * Q],
             a3 = src[j + 3 * Q];
      if (Ns > 1) {
        const int k = j & (Ns - 1);
        a1 = cmul(a1, twid<INV>(tw, k * tstride));
        a2 = cmul(a2, twid<INV>(tw, 2 * k * tstride));
        a3 = cmul(a3, twid<INV>(tw, 3 * k * tstride));
      }
      dft4<INV>(a0, a1, a2, a3);
      v[e][0] = a0; v[e][1] = a1; v[e][2] = a2; v[e][3] = a3;
    }
    __syncthreads();
#pragma unroll
    for (int e = 0; e < PER; ++e) {
      const int b = tid + e * NT;
      const int f = b / Q, j = b % Q;
      const int k = j & (Ns - 1);
      float2 *dst = buf + f * M + (j / Ns) * Ns * 4 + k;
      dst[0] = v[e][0];
      dst[Ns] = v[e][1];
      dst[2 * Ns] = v[e][2];
      dst[3 * Ns] = v[e][3];
    }
    __syncthreads();
    Ns *= 4;
  }
  if (LOG2M & 1) {
    // final radix-2 pass, Ns = M/2: butterfly j pairs (j, j+M/2), twiddle tw[j]
    constexpr int H = M / 2;
    constexpr int BF2 = NB * H;
    constexpr int PER2 = (BF2 + NT - 1) / NT;
    float2 v[PER2][2];
#pragma unroll
    for (int e = 0; e < PER2; ++e) {
      const int b = tid + e * NT;
      if (BF2 % NT == 0 || b < BF2) {
        const int f = b / H, j = b % H;
        const float2 *src = buf + f * M;
        float2 a0 = src[j];
        float2 a1 = cmul(src[j + H], twid<INV>(tw, j));
        v[e][0] = cadd(a0, a1);
        v[e][1] = csub(a0, a1);
      }
    }
    __syncthreads();
#pragma unroll
    for (int e = 0; e < PER2; ++e) {
      const int b = tid + e * NT;
      if (BF2 % NT == 0 || b < BF2) {
        const int f = b / H, j = b % H;
        buf[f * M + j] = v[e][0];
        buf[f * M + j + H] = v[e][1];
      }
    }
    __syncthreads();
  }
}
