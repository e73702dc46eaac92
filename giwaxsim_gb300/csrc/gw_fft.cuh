// Batched mixed-radix complex FFTs in shared memory (Stockham autosort,
// register butterflies of radix 16, 8, 4, 2, 5 and 3).
//
// NB sequences of length M are transformed together by one block.  A pass
// with radix R and stride Ns reads, for butterfly j, the R values
// j + r*(M/R), multiplies value r by exp(-+2 pi i r (j mod Ns) / (Ns R)),
// does an R-point DFT in registers and writes output r to
// (j / Ns) * Ns * R + (j mod Ns) + r * Ns; after the last pass the sequence
// is in natural order.  M = 16^a * R2 * F with R2 in {1,2,4,8} and F in
// {1,3,5}; the passes are a radix-16 passes, then R2, then F, so a
// 2048-point transform is (16, 16, 8) and a 1280-point one (16, 16, 5).
//
// Shared layout: element a of sequence f lives at f*ldm + a + (a >> 4).  With
// that one-in-sixteen padding every pass's reads (consecutive j) and writes
// (stride R when Ns = 1, consecutive otherwise) fall into 16 distinct 8-byte
// bank pairs per half-warp, i.e. no bank conflicts.
//
// Twiddles come from per-pass tables made in float64 on the host:
// tw[k*(R-1) + r-1] = W_{Ns R}^{r k} for even R (lanes read consecutive k at
// the odd stride R-1, conflict-free) and tw[(r-1)*Ns + k] for odd R (lanes
// read consecutive k).  No pass evaluates a transcendental.
//
// The first pass of a transform can read its inputs from a functor (global
// memory) and the last pass can hand its outputs to a functor, so the
// transform's input and output need no shared-memory round trip.
#pragma once

#include "gw_bfly.cuh"
#include "gw_dft.cuh"

__host__ __device__ constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n / 2); }
__host__ __device__ constexpr int fft_pad(int a) { return a + (a >> 4); }
// Values per sequence in the shared-memory FFT buffer of length m.
__host__ __device__ constexpr int fft_ldm(int m) { return fft_pad(m) + 4; }
// odd factor of a supported length (1, 3 or 5)
__host__ __device__ constexpr int fft_odd(int m) { return (m & 1) ? m : fft_odd(m >> 1); }

// Pass plan: a radix-16 passes, then R2 (pow2 remainder), then F (odd).
template <int M>
struct FftPlan {
  static constexpr int F = fft_odd(M);
  static_assert(F == 1 || F == 3 || F == 5, "M = 2^k, 3*2^k or 5*2^k");
  static constexpr int P2 = M / F;
  static constexpr int L2 = ilog2(P2);
  static constexpr int N16 = L2 / 4;                 // radix-16 passes
  static constexpr int R2 = 1 << (L2 - 4 * N16);    // 1 if none
  static constexpr int NPASS = N16 + (R2 > 1) + (F > 1);
  static constexpr int LDM = fft_ldm(M);  // floats2 per sequence (+4: see f-fastest maps)
  // twiddle table length (passes with Ns > 1)
  __host__ __device__ static constexpr int tw_len() {
    int t = 0, ns = 16;
    for (int p = 1; p < N16; ++p) { t += ns * 15; ns *= 16; }
    if (R2 > 1) { t += ns * (R2 - 1); ns *= R2; }
    if (F > 1) t += ns * (F - 1);
    return t > 0 ? t : 1;
  }
  // table offsets of the R2 and F passes
  __host__ __device__ static constexpr int tw_r2() {
    int t = 0, ns = 16;
    for (int p = 1; p < N16; ++p) { t += ns * 15; ns *= 16; }
    return t;
  }
  __host__ __device__ static constexpr int tw_f() {
    return tw_r2() + (R2 > 1 ? (1 << (4 * N16)) * (R2 - 1) : 0);
  }
};

template <int M>
struct FftShape;
// NB sequences per block, NT threads: every thread holds about 16 points
// per pass.  MINB: blocks per SM the register budget is sized for (about
// 1024 threads per SM, i.e. at most 64 registers per thread) so that
// latency is hidden by ~32 resident warps.
template <> struct FftShape<64>   { static constexpr int NB = 16, NT = 64,  MINB = 16; };
template <> struct FftShape<128>  { static constexpr int NB = 16, NT = 128, MINB = 8; };
template <> struct FftShape<256>  { static constexpr int NB = 8,  NT = 128, MINB = 8; };
template <> struct FftShape<384>  { static constexpr int NB = 8,  NT = 192, MINB = 5; };
template <> struct FftShape<512>  { static constexpr int NB = 8,  NT = 256, MINB = 4; };
template <> struct FftShape<640>  { static constexpr int NB = 8,  NT = 320, MINB = 3; };
template <> struct FftShape<768>  { static constexpr int NB = 4,  NT = 192, MINB = 5; };
template <> struct FftShape<1024> { static constexpr int NB = 4,  NT = 256, MINB = 4; };
template <> struct FftShape<1280> { static constexpr int NB = 4,  NT = 320, MINB = 3; };
template <> struct FftShape<1536> { static constexpr int NB = 4,  NT = 384, MINB = 2; };
template <> struct FftShape<2048> { static constexpr int NB = 4,  NT = 512, MINB = 2; };
template <> struct FftShape<2560> { static constexpr int NB = 2,  NT = 320, MINB = 3; };
template <> struct FftShape<3072> { static constexpr int NB = 2,  NT = 384, MINB = 2; };
template <> struct FftShape<4096> { static constexpr int NB = 2,  NT = 512, MINB = 2; };
template <> struct FftShape<5120> { static constexpr int NB = 1,  NT = 320, MINB = 3; };
template <> struct FftShape<6144> { static constexpr int NB = 1,  NT = 384, MINB = 2; };
template <> struct FftShape<8192> { static constexpr int NB = 1,  NT = 512, MINB = 1; };

// Blocks per SM the pruned row kernels (window and band within M/2) are
// sized for: their 1280-point form fits four 320-thread blocks in 48
// registers without spills (measured 10 % faster than three); the other
// lengths keep MINB.
template <int M>
__host__ __device__ constexpr int minb_pruned_rows() {
  return M == 1280 ? 4 : FftShape<M>::MINB;
}

// The supported lengths, ascending.
constexpr int kFftSizes[] = {64, 128, 256, 384, 512, 640, 768, 1024, 1280,
                             1536, 2048, 2560, 3072, 4096, 5120, 6144, 8192};

// Twiddle-table offset of radix-16 pass p (p >= 1) of a length-M plan.
template <int M>
__host__ __device__ constexpr int tw_offset(int p) {
  int t = 0, ns = 16;
  for (int q = 1; q < p; ++q) { t += ns * 15; ns *= 16; }
  return t;
}

// Generic pass.  SRC: 0 = shared memory (optionally multiplied by pre[n]),
// 1 = load(f, n).  DST: 0 = shared memory, 1 = store(f, m, value).
// FFAST maps the sequence index f fastest across threads (column loads from
// global memory); otherwise the butterfly index j is fastest.
// Pruning (the chirp-z window and band are shorter than M): HIN, in a first
// pass (NS = 1), reads only the inputs r < R/2 of each butterfly (the
// others, n >= M/2, are zero) and transforms them with the pruned register
// DFT; HOUT, in a last pass, produces only the outputs r < ceil(R/2) (the
// others, m >= M/2, are not wanted), the rest being dead code.
template <int M, int R, int NS, int NB, int NT, bool INV, int SRC, bool PREMUL,
          int DST, bool FFAST, bool HIN = false, bool HOUT = false, class Load,
          class Store>
__device__ __forceinline__ void fft_pass(float2 *buf, const float2 *tw,
                                         const float2 *pre, Load load,
                                         Store store) {
  static_assert(!HIN || NS == 1, "input pruning is for a first pass");
  constexpr int KIN = HIN ? R / 2 : R, KOUT = HOUT ? (R + 1) / 2 : R;
  constexpr int Q = M / R;
  constexpr int BF = NB * Q;
  constexpr int PER = (BF + NT - 1) / NT;
  constexpr int LDM = FftPlan<M>::LDM;
  float2 v[PER][R];
#pragma unroll
  for (int e = 0; e < PER; ++e) {
    const int b = threadIdx.x + e * NT;
    if (BF % NT == 0 || b < BF) {
      const int f = FFAST ? b % NB : b / Q;
      const int j = FFAST ? b / NB : b % Q;
      // with Q a multiple of 16, fft_pad(j + r Q) = fft_pad(j) + r (Q + Q/16):
      // one address per butterfly and compile-time offsets
      const float2 *src = buf + f * LDM + fft_pad(j);
#pragma unroll
      for (int r = 0; r < KIN; ++r) {
        const int n = j + r * Q;
        if (SRC == 0) {
          float2 x = Q % 16 == 0 ? src[r * (Q + Q / 16)] : buf[f * LDM + fft_pad(n)];
          if (PREMUL) x = cmul(x, __ldg(pre + n));
          v[e][r] = x;
        } else {
          v[e][r] = load(f, n);
        }
      }
      if (NS > 1) {
        const int k = j % NS;
        if constexpr (R & 1) {
#pragma unroll
          for (int r = 1; r < R; ++r)
            v[e][r] = cmul(v[e][r], conj_if<INV>(tw[(r - 1) * NS + k]));
        } else {
          const float2 *t = tw + k * (R - 1) - 1;
#pragma unroll
          for (int r = 1; r < R; ++r) v[e][r] = cmul(v[e][r], conj_if<INV>(t[r]));
        }
      }
      if constexpr (HIN) gwd::dft_prefix<R, KIN, INV>(v[e]);
      else dft<R, INV>(v[e]);
    }
  }
  // The writes wait for every thread's reads (passes are in place; a first
  // pass may read inputs that alias its shared destination), except in a
  // last pass (NS R = M): there Q = NS, so base = j and a butterfly writes
  // exactly the slots j + r Q it read, which no other thread touches.
  constexpr bool kOwnSlots = NS * R == M && SRC == 0;
  if (DST == 0 && !kOwnSlots) __syncthreads();
#pragma unroll
  for (int e = 0; e < PER; ++e) {
    const int b = threadIdx.x + e * NT;
    if (BF % NT == 0 || b < BF) {
      const int f = FFAST ? b % NB : b / Q;
      const int j = FFAST ? b / NB : b % Q;
      const int k = j % NS;
      const int base = (j / NS) * NS * R + k;
      // NS a multiple of 16: fft_pad(base + r NS) = fft_pad(base) + r (NS + NS/16);
      // NS = 1 and R <= 16 with base = j R a multiple of 16 (R = 16): + r
      constexpr bool kStride = NS % 16 == 0 || (NS == 1 && R == 16);
      constexpr int kStep = NS == 1 ? 1 : NS + NS / 16;
      float2 *dst = buf + f * LDM + fft_pad(base);
#pragma unroll
      for (int r = 0; r < KOUT; ++r) {
        const int m = base + r * NS;
        // dft_prefix leaves natural order, dft its out_slot order
        const float2 val = HIN ? v[e][r] : v[e][out_slot<R>(r)];
        if (DST == 0) {
          if (kStride) dst[r * kStep] = val;
          else buf[f * LDM + fft_pad(m)] = val;
        } else {
          store(f, m, val);
        }
      }
    }
  }
  if (DST == 0) __syncthreads();
}

struct NoLoad {
  __device__ float2 operator()(int, int) const { return make_float2(0.f, 0.f); }
};
struct NoStore {
  __device__ void operator()(int, int, float2) const {}
};

// Whole transform.  The first pass reads shared memory (SRC=0, times pre[n]
// when PREMUL) or load(f, n) (SRC=1); the last pass writes shared memory
// (DST=0) or calls store(f, m, value) (DST=1).  Middle passes stay in shared
// memory.  A transform ending in shared memory leaves the block synchronised.
// HIN / HOUT: the first pass reads only the first half of its inputs / the
// last pass produces only the first half of its outputs (fft_pass).
template <int M, int NB, int NT, bool INV, int SRC, bool PREMUL, int DST,
          bool FFAST_FIRST, bool HIN = false, bool HOUT = false, class Load,
          class Store>
__device__ __forceinline__ void fft_run(float2 *buf, const float2 *tw,
                                        const float2 *pre, Load load,
                                        Store store) {
  using Pl = FftPlan<M>;
  static_assert(Pl::N16 >= 1, "M >= 16");
  if constexpr (Pl::NPASS == 1) {
    fft_pass<M, 16, 1, NB, NT, INV, SRC, PREMUL, DST, FFAST_FIRST, HIN, HOUT>(
        buf, tw, pre, load, store);
  } else {
    fft_pass<M, 16, 1, NB, NT, INV, SRC, PREMUL, 0, FFAST_FIRST, HIN, false>(
        buf, tw, pre, load, NoStore());
    if constexpr (Pl::N16 >= 2) {
      constexpr int dst = Pl::NPASS == 2 ? DST : 0;
      fft_pass<M, 16, 16, NB, NT, INV, 0, false, dst, false, false,
               HOUT && Pl::NPASS == 2>(buf, tw + tw_offset<M>(1), nullptr, NoLoad(), store);
    }
    if constexpr (Pl::N16 >= 3) {
      constexpr int dst = Pl::NPASS == 3 ? DST : 0;
      fft_pass<M, 16, 256, NB, NT, INV, 0, false, dst, false, false,
               HOUT && Pl::NPASS == 3>(buf, tw + tw_offset<M>(2), nullptr, NoLoad(), store);
    }
    if constexpr (Pl::R2 > 1) {
      constexpr int NS2 = 1 << (4 * Pl::N16);
      constexpr int dst = Pl::F == 1 ? DST : 0;
      fft_pass<M, Pl::R2, NS2, NB, NT, INV, 0, false, dst, false, false,
               HOUT && Pl::F == 1>(buf, tw + Pl::tw_r2(), nullptr, NoLoad(), store);
    }
    if constexpr (Pl::F > 1) {
      fft_pass<M, Pl::F, Pl::P2, NB, NT, INV, 0, false, DST, false, false, HOUT>(
          buf, tw + Pl::tw_f(), nullptr, NoLoad(), store);
    }
  }
}
