// Register DFTs of compile-time length for the fused chirp-z kernels.
//
// dft_ip<R, INV, KA, MAP>(v) transforms R values held by one thread in
// place, X[k] = sum_n x[n] W_R^{n k} with W_R = exp(-+2 pi i / R) (forward
// minus, inverse plus, no scaling).  Only x[0..KA) are read: the others are
// taken as zero and the butterflies that would add those zeros are left out
// (input pruning; a compiler cannot drop them itself, because x + 0.0f is
// not x for x = -0.0f).  Outputs that the caller never uses are removed by
// dead-code elimination, so output pruning needs no code.
//
// Lengths: 2, 3, 4, 5, 8, 16 directly (gw_bfly.cuh's butterflies), and
// R = P * Q in two stages for 12, 20, 24, 32, 40, 48 (n = Q a + b,
// k = c + P d: Q DFTs of length P over a, twiddles W_R^{b c}, P DFTs of
// length Q over b).  Every twiddle is a compile-time constant: cos and sin of
// 2 pi e / R evaluated in double by Taylor series after an exact octant
// reduction of the rational angle, then rounded to float.
#pragma once

#include <utility>

#include "gw_bfly.cuh"

namespace gwd {

// ------------------------------------------------------- constant trig
// sin and cos of x for |x| <= pi/4 by their Taylor series (terms beyond x^25
// are below 1e-27 there).
__host__ __device__ constexpr double taylor_sin(double x) {
  double term = x, sum = x;
  for (int k = 1; k <= 12; ++k) {
    term *= -x * x / ((2.0 * k) * (2.0 * k + 1.0));
    sum += term;
  }
  return sum;
}
__host__ __device__ constexpr double taylor_cos(double x) {
  double term = 1.0, sum = 1.0;
  for (int k = 1; k <= 12; ++k) {
    term *= -x * x / ((2.0 * k - 1.0) * (2.0 * k));
    sum += term;
  }
  return sum;
}

// cos(2 pi e / n) (want_sin false) or sin(2 pi e / n): the angle is
// (pi/4)(o + v) with octant o = floor(8 e' / n) and v in [0, 1) (e' = e mod
// n, exact integers); each octant maps to cos or sin of (pi/4) v or of
// (pi/4)(1 - v), both within [0, pi/4].
__host__ __device__ constexpr double trig2pi(long long e, long long n,
                                             bool want_sin) {
  constexpr double kPi4 = 0.78539816339744830962;
  long long r = e % n;
  if (r < 0) r += n;
  const long long q = 8 * r;
  const long long o = q / n, rem = q - o * n;
  const double v = (double)rem / (double)n;
  const double w = (double)(n - rem) / (double)n;
  const double Cv = taylor_cos(kPi4 * v), Sv = taylor_sin(kPi4 * v);
  const double Cw = taylor_cos(kPi4 * w), Sw = taylor_sin(kPi4 * w);
  double c = 0.0, s = 0.0;
  switch (o) {
    case 0: c = Cv; s = Sv; break;
    case 1: c = Sw; s = Cw; break;
    case 2: c = -Sv; s = Cv; break;
    case 3: c = -Cw; s = Sw; break;
    case 4: c = -Cv; s = -Sv; break;
    case 5: c = -Sw; s = -Cw; break;
    case 6: c = Sv; s = -Cv; break;
    default: c = Cw; s = -Sw; break;
  }
  return want_sin ? s : c;
}

// ----------------------------------------------------- static for
// A compile-time int usable in device code (std::integral_constant's
// conversion is host-only under nvcc).
template <int I>
struct Ic {
  static constexpr int value = I;
  __host__ __device__ constexpr operator int() const { return I; }
};

template <class F, int... I>
__host__ __device__ __forceinline__ void sfor_seq(F &&f, std::integer_sequence<int, I...>) {
  (f(Ic<I>{}), ...);
}
// f(Ic<0>), ..., f(Ic<N-1>): a fully unrolled loop whose index is a
// constant expression in the body
template <int N, class F>
__host__ __device__ __forceinline__ void sfor(F &&f) {
  sfor_seq(f, std::make_integer_sequence<int, N>{});
}

// ------------------------------------------------------- twiddles
// v * W_R^E (forward, W_R = exp(-2 pi i / R)) or v * conj(W_R^E) (inverse).
template <int E, int R, bool INV>
__host__ __device__ __forceinline__ float2 twmul(float2 v) {
  constexpr int e = ((E % R) + R) % R;
  if constexpr (e == 0) {
    return v;
  } else if constexpr (2 * e == R) {
    return make_float2(-v.x, -v.y);
  } else if constexpr (4 * e == R) {  // W = -i
    return INV ? make_float2(-v.y, v.x) : make_float2(v.y, -v.x);
  } else if constexpr (4 * e == 3 * R) {  // W = +i
    return INV ? make_float2(v.y, -v.x) : make_float2(-v.y, v.x);
  } else {
    constexpr float c = (float)trig2pi(e, R, false);
    constexpr float s = (float)trig2pi(e, R, true);
    // forward W = c - i s; inverse conj(W) = c + i s
    constexpr float t = INV ? s : -s;
    return make_float2(v.x * c - v.y * t, v.x * t + v.y * c);
  }
}

// ------------------------------------------------- base-case DFTs
// Full DFT of a base length in natural output order.
template <int R, bool INV>
__host__ __device__ __forceinline__ void dft_base(float2 (&u)[R]) {
  float2 v[R];
  sfor<R>([&](auto i) { v[i] = u[i]; });
  dft<R, INV>(v);
  sfor<R>([&](auto k) { u[k] = v[out_slot<R>(k)]; });
}

// DFT of length P whose inputs u[a] for a >= NA are zero (and not read),
// natural output order.
template <int P, int NA, bool INV>
__host__ __device__ __forceinline__ void dft_prefix(float2 (&u)[P]) {
  static_assert(NA >= 1 && NA <= P, "nonzero input count");
  if constexpr (NA == P) {
    dft_base<P, INV>(u);
  } else if constexpr (NA == 1) {
    sfor<P>([&](auto c) { u[c] = u[0]; });
  } else if constexpr (P == 8 && NA <= 4) {
    // X[2c'] = DFT4(u)[c'], X[2c'+1] = DFT4(u[a] W_8^a)[c']
    float2 e[4], o[4];
    sfor<4>([&](auto a) {
      if constexpr (a < NA) {
        e[a] = u[a];
        o[a] = twmul<a, 8, INV>(u[a]);
      } else {
        e[a] = make_float2(0.f, 0.f);
        o[a] = make_float2(0.f, 0.f);
      }
    });
    dft4<INV>(e[0], e[1], e[2], e[3]);
    dft4<INV>(o[0], o[1], o[2], o[3]);
    sfor<4>([&](auto c) {
      u[2 * c] = e[c];
      u[2 * c + 1] = o[c];
    });
  } else if constexpr (P == 16 && NA <= 8) {
    // X[2c'] = DFT8(u)[c'], X[2c'+1] = DFT8(u[a] W_16^a)[c']
    float2 e[8], o[8];
    sfor<8>([&](auto a) {
      if constexpr (a < NA) {
        e[a] = u[a];
        o[a] = twmul<a, 16, INV>(u[a]);
      }
    });
    dft_prefix<8, (NA < 8 ? NA : 8), INV>(e);
    dft_prefix<8, (NA < 8 ? NA : 8), INV>(o);
    sfor<8>([&](auto c) {
      u[2 * c] = e[c];
      u[2 * c + 1] = o[c];
    });
  } else {
    // direct sum over the nonzero inputs
    float2 X[P];
    sfor<P>([&](auto c) {
      float2 acc = u[0];
      sfor<NA - 1>([&](auto am1) {
        constexpr int a = am1 + 1;
        acc = cadd(acc, twmul<a * c, P, INV>(u[a]));
      });
      X[c] = acc;
    });
    sfor<P>([&](auto c) { u[c] = X[c]; });
  }
}

// Two-stage split of a composite length: P (over a, n = Q a + b) times Q.
template <int R> struct Split;
template <> struct Split<12> { static constexpr int P = 4, Q = 3; };
template <> struct Split<20> { static constexpr int P = 4, Q = 5; };
template <> struct Split<24> { static constexpr int P = 8, Q = 3; };
template <> struct Split<32> { static constexpr int P = 8, Q = 4; };
template <> struct Split<40> { static constexpr int P = 8, Q = 5; };
template <> struct Split<48> { static constexpr int P = 16, Q = 3; };

template <int R>
__host__ __device__ constexpr bool is_base() {
  return R == 2 || R == 3 || R == 4 || R == 5 || R == 8 || R == 16;
}

// ------------------------------------------------- in-place transforms
// dft_ip<R, INV, KA, MAP>(v): the DFT of x[0..R) computed in place in v,
// with input x[n] held in slot in_slot<R, MAP>(n) (MAP 0: slot n; MAP 1:
// slot pslot<R>(n), the order this transform leaves its outputs in) and
// output X[k] left in slot out_at<R, MAP>(k) = in_slot<R, MAP>(pslot<R>(k)).
// Each stage works on one group of slots at a time and writes its results
// back into the same slots, so no more than R values (plus one group) are
// live at once; all slot arithmetic is compile-time, so orders cost
// nothing.  For a composite R = P * Q (n = Q a + b, k = c + P d), stage A
// turns the group {Q a + b : a} of each b into {Q c + b : c} and stage B the
// group {Q c + b : b} of each c into {Q c + d : d}: X[c + P d] sits in slot
// Q c + d, i.e. pslot(k) = Q (k mod P) + k div P.  Base lengths are
// transformed on a temporary and written back in natural order.
template <int R>
__host__ __device__ constexpr int pslot(int k) {
  if constexpr (is_base<R>()) {
    return k;
  } else {
    return Split<R>::Q * (k % Split<R>::P) + k / Split<R>::P;
  }
}

template <int R, int MAP>
__host__ __device__ constexpr int in_slot(int n) {
  return MAP == 0 ? n : pslot<R>(n);
}

// Slot of output k of dft_ip<R, INV, KA, MAP>.
template <int R, int MAP>
__host__ __device__ constexpr int out_at(int k) {
  return in_slot<R, MAP>(pslot<R>(k));
}

template <int R, bool INV, int KA = R, int MAP = 0>
__host__ __device__ __forceinline__ void dft_ip(float2 (&v)[R]) {
  static_assert(KA >= 1 && KA <= R, "nonzero input count");
  if constexpr (is_base<R>()) {
    float2 u[R];
    sfor<KA>([&](auto n) { u[n] = v[in_slot<R, MAP>(n)]; });
    dft_prefix<R, KA, INV>(u);
    sfor<R>([&](auto k) { v[in_slot<R, MAP>(k)] = u[k]; });
  } else {
    constexpr int P = Split<R>::P, Q = Split<R>::Q;
    // stage A: for each b, the P-point DFTs over a, twiddled by W_R^{b c}
    sfor<Q>([&](auto b) {
      constexpr int NA0 = (KA - b + Q - 1) / Q;
      constexpr int NA = NA0 < 1 ? 1 : (NA0 > P ? P : NA0);
      float2 u[P];
      sfor<P>([&](auto a) {
        if constexpr (a < NA) {
          if constexpr (Q * a + b < KA) u[a] = v[in_slot<R, MAP>(Q * a + b)];
          else u[a] = make_float2(0.f, 0.f);
        }
      });
      dft_prefix<P, NA, INV>(u);
      sfor<P>([&](auto c) { v[in_slot<R, MAP>(Q * c + b)] = twmul<b * c, R, INV>(u[c]); });
    });
    // stage B: for each c, the Q-point DFT over b
    sfor<P>([&](auto c) {
      float2 w[Q];
      sfor<Q>([&](auto b) { w[b] = v[in_slot<R, MAP>(Q * c + b)]; });
      dft_base<Q, INV>(w);
      sfor<Q>([&](auto d) { v[in_slot<R, MAP>(Q * c + d)] = w[d]; });
    });
  }
}

}  // namespace gwd
