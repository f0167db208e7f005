// Line-FFT engine for sm_103a: Stockham autosort stages with in-register
// radix codelets, shared-memory exchanges between stages, and compile-time
// radix plans.  Every pass kernel of the library (contiguous z lines, strided
// y/x columns) is built from LineFFT<T, L>::run().
//
// Conventions
//   * All codelets and stage twiddles compute the FORWARD transform
//     X[k] = sum_n x[n] exp(-2*pi*i*n*k/L)  (FFTW/cuFFT sign -1, unnormalised).
//     Inverse passes use conj(FFT(conj(x))) : the pass kernels conjugate on
//     load and on store, so one engine serves both directions.
//   * A line of length L is processed by P = L/E threads, each holding E
//     complex values in registers.  Stage 0 has radix E (one butterfly per
//     thread) and reads its inputs straight from the caller's loader; the
//     last stage hands its outputs straight to the caller's storer, so a
//     pass touches HBM exactly once each way.
//   * Stage s (radix R, sub-transform size Ns = product of earlier radices)
//     reads x[j + r*L/R] and writes y[(j/Ns)*Ns*R + j%Ns + r*Ns] after the
//     twiddle w_{Ns*R}^{(j%Ns)*r}.  This is the textbook Stockham
//     formulation (natural-order output, no bit reversal).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <type_traits>
#include "df64.cuh"
#include "line_plan.h"

namespace afg {

// ---------------------------------------------------------------- complex
// CT<T>::V is the complex type the arithmetic runs in (registers, shared
// memory, twiddle tables); Mem<T> the real and complex types of the arrays in
// global memory.  They differ only for double-float (IEEE double arrays).
template <typename T> struct CT;
template <> struct CT<float>  { typedef float2  V; };
template <> struct CT<double> { typedef double2 V; };
template <> struct CT<df>     { typedef dfc     V; };
template <typename T> struct Mem { typedef T R; typedef typename CT<T>::V C; };
template <> struct Mem<df> { typedef double R; typedef double2 C; };

// array element -> arithmetic type and back (identity but for double-float,
// which scales by 2^sh on the way in and 2^-sh on the way out)
template <typename T> __device__ __forceinline__ typename CT<T>::V to_reg(int, typename Mem<T>::C m) { return m; }
template <> __device__ __forceinline__ dfc to_reg<df>(int sh, double2 m) {
  return dfc{df_from_double(m.x, sh), df_from_double(m.y, sh)};
}
template <typename T> __device__ __forceinline__ typename Mem<T>::C to_mem(int, typename CT<T>::V v) { return v; }
template <> __device__ __forceinline__ double2 to_mem<df>(int sh, dfc v) {
  return make_double2(df_to_double(v.x, sh), df_to_double(v.y, sh));
}
// a pass's scale exponent (double-float: from the transform's input exponent)
template <typename T> __device__ __forceinline__ int pass_shift(const int*) { return 0; }
template <> __device__ __forceinline__ int pass_shift<df>(const int* dfx) { return df_shift_of(__ldg(dfx)); }
// twiddle-table entry through the read-only path
__device__ __forceinline__ float2 ld_tw(const float2* p) { return __ldg(p); }
__device__ __forceinline__ double2 ld_tw(const double2* p) { return __ldg(p); }
__device__ __forceinline__ dfc ld_tw(const dfc* p) {
  const float4 f = __ldg(reinterpret_cast<const float4*>(p));
  return dfc{df_make(f.x, f.y), df_make(f.z, f.w)};
}

template <typename V> __device__ __forceinline__ V c_add(V a, V b) { V r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename V> __device__ __forceinline__ V c_sub(V a, V b) { V r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename V> __device__ __forceinline__ V c_mul(V a, V b) {
  V r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
// a * (-i)
template <typename V> __device__ __forceinline__ V c_mmi(V a) { V r; r.x = a.y; r.y = -a.x; return r; }
template <typename V> __device__ __forceinline__ V c_conj(V a) { V r; r.x = a.x; r.y = -a.y; return r; }
template <typename V, typename S> __device__ __forceinline__ V c_scale(V a, S s) { V r; r.x = a.x * s; r.y = a.y * s; return r; }
template <typename V> __device__ __forceinline__ V c_make(decltype(V().x) x, decltype(V().x) y) { V r; r.x = x; r.y = y; return r; }

// ------------------------------------------------- compile-time trigonometry
// cos/sin(2*pi*n/d) for integer n, d evaluated as constant expressions.
// Octant reduction with exact integer arithmetic, then Maclaurin series on
// [0, pi/4] (22 terms: far below double rounding there).
__host__ __device__ constexpr double ce_pi() { return 3.14159265358979323846264338327950288; }
__host__ __device__ constexpr double ce_sin_q(double x) {
  double x2 = x * x, term = x, sum = x;
  for (int k = 1; k < 22; ++k) { term *= -x2 / double((2 * k) * (2 * k + 1)); sum += term; }
  return sum;
}
__host__ __device__ constexpr double ce_cos_q(double x) {
  double x2 = x * x, term = 1.0, sum = 1.0;
  for (int k = 1; k < 22; ++k) { term *= -x2 / double((2 * k - 1) * (2 * k)); sum += term; }
  return sum;
}
// returns cos (want_sin = false) or sin (want_sin = true) of 2*pi*n/d
__host__ __device__ constexpr double ce_trig2pi(long long n, long long d, bool want_sin) {
  long long m = n % d; if (m < 0) m += d;
  long long o = (8 * m) / d;            // octant 0..7
  long long r = 8 * m - o * d;          // 0 <= r < d
  double phi = (ce_pi() / 4.0) * (double(r) / double(d));
  double psi = (ce_pi() / 4.0) * (double(d - r) / double(d));
  double c = 0, s = 0;
  switch (o) {
    case 0: c = ce_cos_q(phi);  s = ce_sin_q(phi);  break;
    case 1: c = ce_sin_q(psi);  s = ce_cos_q(psi);  break;
    case 2: c = -ce_sin_q(phi); s = ce_cos_q(phi);  break;
    case 3: c = -ce_cos_q(psi); s = ce_sin_q(psi);  break;
    case 4: c = -ce_cos_q(phi); s = -ce_sin_q(phi); break;
    case 5: c = -ce_sin_q(psi); s = -ce_cos_q(psi); break;
    case 6: c = ce_sin_q(phi);  s = -ce_cos_q(phi); break;
    default: c = ce_cos_q(psi); s = -ce_sin_q(psi); break;
  }
  return want_sin ? s : c;
}

template <int B, int E, typename F>
__device__ __forceinline__ void static_for(F&& f) {
  if constexpr (B < E) {
    f(std::integral_constant<int, B>{});
    static_for<B + 1, E>(f);
  }
}

// multiply by the constant w_R^m = exp(-2*pi*i*m/R)
template <int R, int M, typename V>
__device__ __forceinline__ V c_mul_w(V a) {
  typedef decltype(V().x) T;
  constexpr int m = ((M % R) + R) % R;
  if constexpr (m == 0) {
    return a;
  } else if constexpr (4 * m == R) {          // -i
    return c_mmi(a);
  } else if constexpr (2 * m == R) {          // -1
    return c_make<V>(-a.x, -a.y);
  } else if constexpr (4 * m == 3 * R) {      // +i
    return c_make<V>(-a.y, a.x);
  } else {
    constexpr T c = T(ce_trig2pi(m, R, false));
    constexpr T s = T(-ce_trig2pi(m, R, true));   // imaginary part of w
    return c_make<V>(a.x * c - a.y * s, a.x * s + a.y * c);
  }
}

// ------------------------------------------------------------------ codelets
// Dft<R, S>::run(v): in-place forward DFT of v[0], v[S], ..., v[(R-1)S].
template <int R, int S> struct Dft;

template <int S> struct Dft<1, S> { template <typename V> __device__ __forceinline__ static void run(V*) {} };

template <int S> struct Dft<2, S> {
  template <typename V> __device__ __forceinline__ static void run(V* v) {
    V a = v[0], b = v[S];
    v[0] = c_add(a, b); v[S] = c_sub(a, b);
  }
};

template <int S> struct Dft<3, S> {
  template <typename V> __device__ __forceinline__ static void run(V* v) {
    typedef decltype(V().x) T;
    constexpr T h = T(0.866025403784438646763723170752936183);   // sin(pi/3)
    V t = c_add(v[S], v[2 * S]);
    V d = c_sub(v[S], v[2 * S]);
    V m = c_make<V>(v[0].x - T(0.5) * t.x, v[0].y - T(0.5) * t.y);
    v[0] = c_add(v[0], t);
    V q = c_make<V>(d.y * h, -d.x * h);                          // -i*h*d
    v[S] = c_add(m, q); v[2 * S] = c_sub(m, q);
  }
};

template <int S> struct Dft<4, S> {
  template <typename V> __device__ __forceinline__ static void run(V* v) {
    V t0 = c_add(v[0], v[2 * S]), t1 = c_sub(v[0], v[2 * S]);
    V t2 = c_add(v[S], v[3 * S]), t3 = c_mmi(c_sub(v[S], v[3 * S]));
    v[0] = c_add(t0, t2); v[2 * S] = c_sub(t0, t2);
    v[S] = c_add(t1, t3); v[3 * S] = c_sub(t1, t3);
  }
};

template <int S> struct Dft<5, S> {
  template <typename V> __device__ __forceinline__ static void run(V* v) {
    typedef decltype(V().x) T;
    constexpr T c1 = T(0.309016994374947424102293417182819059);    // cos(2pi/5)
    constexpr T c2 = T(-0.809016994374947424102293417182819059);   // cos(4pi/5)
    constexpr T s1 = T(0.951056516295153572116439333379382143);    // sin(2pi/5)
    constexpr T s2 = T(0.587785252292473129168705954639072769);    // sin(4pi/5)
    V b1 = c_add(v[S], v[4 * S]), d1 = c_sub(v[S], v[4 * S]);
    V b2 = c_add(v[2 * S], v[3 * S]), d2 = c_sub(v[2 * S], v[3 * S]);
    V x0 = v[0];
    V r1 = c_make<V>(x0.x + c1 * b1.x + c2 * b2.x, x0.y + c1 * b1.y + c2 * b2.y);
    V r2 = c_make<V>(x0.x + c2 * b1.x + c1 * b2.x, x0.y + c2 * b1.y + c1 * b2.y);
    V i1 = c_make<V>(s1 * d1.x + s2 * d2.x, s1 * d1.y + s2 * d2.y);
    V i2 = c_make<V>(s2 * d1.x - s1 * d2.x, s2 * d1.y - s1 * d2.y);
    v[0] = c_add(x0, c_add(b1, b2));
    V q1 = c_mmi(i1), q2 = c_mmi(i2);
    v[S] = c_add(r1, q1); v[4 * S] = c_sub(r1, q1);
    v[2 * S] = c_add(r2, q2); v[3 * S] = c_sub(r2, q2);
  }
};

template <int S> struct Dft<8, S> {
  template <typename V> __device__ __forceinline__ static void run(V* v) {
    typedef decltype(V().x) T;
    constexpr T h = T(0.707106781186547524400844362104849039);
    Dft<4, 2 * S>::run(v);        // even samples
    Dft<4, 2 * S>::run(v + S);    // odd samples
    V e0 = v[0], e1 = v[2 * S], e2 = v[4 * S], e3 = v[6 * S];
    V o0 = v[S], o1 = v[3 * S], o2 = v[5 * S], o3 = v[7 * S];
    V w1 = c_make<V>(h * (o1.x + o1.y), h * (o1.y - o1.x));    // (1-i)/sqrt2
    V w2 = c_mmi(o2);
    V w3 = c_make<V>(h * (o3.y - o3.x), -h * (o3.x + o3.y));   // (-1-i)/sqrt2
    v[0] = c_add(e0, o0); v[4 * S] = c_sub(e0, o0);
    v[S] = c_add(e1, w1); v[5 * S] = c_sub(e1, w1);
    v[2 * S] = c_add(e2, w2); v[6 * S] = c_sub(e2, w2);
    v[3 * S] = c_add(e3, w3); v[7 * S] = c_sub(e3, w3);
  }
};

__host__ __device__ constexpr int first_factor(int R) {
  return (R % 8 == 0 && R >= 32) ? 8 : (R % 4 == 0) ? 4 : (R % 2 == 0) ? 2 : (R % 3 == 0) ? 3
       : (R % 5 == 0) ? 5 : (R % 7 == 0) ? 7 : R;
}

// Prime (or otherwise unsplit) lengths: direct DFT with conjugate-pair folding.
template <int R, int S> struct DftPrime {
  template <typename V> __device__ __forceinline__ static void run(V* v) {
    typedef decltype(V().x) T;
    constexpr int H = (R - 1) / 2;
    V a[H + 1], b[H + 1];
#pragma unroll
    for (int n = 1; n <= H; ++n) { a[n] = c_add(v[n * S], v[(R - n) * S]); b[n] = c_sub(v[n * S], v[(R - n) * S]); }
    V out[R];
    V x0 = v[0];
    V sum = x0;
#pragma unroll
    for (int n = 1; n <= H; ++n) sum = c_add(sum, a[n]);
    out[0] = sum;
    static_for<1, H + 1>([&](auto k_) {
      constexpr int k = decltype(k_)::value;
      V re = x0, im = c_make<V>(T(0), T(0));
      static_for<1, H + 1>([&](auto n_) {
        constexpr int n = decltype(n_)::value;
        constexpr T c = T(ce_trig2pi((long long)n * k, R, false));
        constexpr T s = T(ce_trig2pi((long long)n * k, R, true));
        re.x += c * a[n].x; re.y += c * a[n].y;
        im.x += s * b[n].x; im.y += s * b[n].y;
      });
      V q = c_mmi(im);                // -i * sum s*b
      out[k] = c_add(re, q); out[R - k] = c_sub(re, q);
    });
#pragma unroll
    for (int n = 0; n < R; ++n) v[n * S] = out[n];
  }
};

// Composite lengths R = A*B: in-register Cooley-Tukey
//   X[k1 + A*k2] = sum_n2 w_B^{n2 k2} w_R^{n2 k1} sum_n1 x[B*n1 + n2] w_A^{n1 k1}
template <int R, int S> struct Dft {
  static constexpr int A = first_factor(R);
  static constexpr int B = R / A;
  template <typename V> __device__ __forceinline__ static void run(V* v) {
    if constexpr (B == 1) {
      DftPrime<R, S>::run(v);
    } else {
      static_for<0, B>([&](auto n2_) { Dft<A, B * S>::run(v + decltype(n2_)::value * S); });
      static_for<1, A>([&](auto k1_) {
        constexpr int k1 = decltype(k1_)::value;
        static_for<1, B>([&](auto n2_) {
          constexpr int n2 = decltype(n2_)::value;
          v[(B * k1 + n2) * S] = c_mul_w<R, n2 * k1>(v[(B * k1 + n2) * S]);
        });
      });
      static_for<0, A>([&](auto k1_) { Dft<B, S>::run(v + B * decltype(k1_)::value * S); });
      V tmp[R];
#pragma unroll
      for (int k1 = 0; k1 < A; ++k1)
#pragma unroll
        for (int k2 = 0; k2 < B; ++k2) tmp[k1 + A * k2] = v[(B * k1 + k2) * S];
#pragma unroll
      for (int i = 0; i < R; ++i) v[i * S] = tmp[i];
    }
  }
};

// EF != 0 forces the first radix (tuning sweeps); 0 selects plan_for()
template <typename T, int L, int EF = 0>
struct LineFFT {
  typedef typename CT<T>::V V;
  static constexpr LinePlan pl = plan_select(L, std::is_same<T, df>::value ? 2 : (sizeof(T) == 8 ? 1 : 0), EF);
  static constexpr int E = pl.E;
  static constexpr int P = pl.P;
  static constexpr int NS = pl.ns;
  static_assert(E > 0, "no radix plan for this length");

  // compute(): every stage of the line transform, outputs left in v[] with
  // the last stage's position mapping (emit() hands them to a storer).
  //   load(p)      stage-0 input at line position p (global or shared memory)
  //   xw/xr        shared-memory exchange accessors of this line
  //   after_load() runs once the stage-0 loads are issued and before the first
  //                exchange overwrites shared memory (a barrier when the loads
  //                read shared memory; a cluster barrier when they read another
  //                CTA's shared memory)
  template <class Load, class XW, class XR, class AfterLoad>
  __device__ __forceinline__ static void compute(int t, const V* __restrict__ tw, Load&& load, XW&& xw, XR&& xr,
                                                 AfterLoad&& after_load, V (&v)[E]) {
#pragma unroll
    for (int r = 0; r < E; ++r) v[r] = load(t + r * P);
    after_load();
    stages(t, tw, xw, xr, [] {}, v);
  }

  // every stage on inputs already in v[r] = x[t + r*P] (stage-0 order);
  // before_exchange() runs once before the first shared-memory exchange
  template <class XW, class XR, class Sync>
  __device__ __forceinline__ static void stages(int t, const V* __restrict__ tw, XW&& xw, XR&& xr,
                                                Sync&& before_exchange, V (&v)[E]) {
    if constexpr (NS >= 1) Dft<E, 1>::run(v);
    if constexpr (NS >= 2) {
      before_exchange();
      static_for<1, NS>([&](auto s_) {
        constexpr int s = decltype(s_)::value;
        constexpr int Rp = pl.radix[s - 1];
        constexpr int R = pl.radix[s];
        constexpr int Nsp = plan_ns_before(pl, s - 1);
        constexpr int Ns = plan_ns_before(pl, s);
        constexpr int two = plan_tw_offset(pl, s);
#pragma unroll
        for (int b = 0; b < E / Rp; ++b) {
          const int j = t + b * P;
          const int base = (j / Nsp) * Nsp * Rp + (j % Nsp);
#pragma unroll
          for (int r = 0; r < Rp; ++r) xw(base + r * Nsp, v[b * Rp + r]);
        }
        __syncthreads();
#pragma unroll
        for (int b = 0; b < E / R; ++b) {
          const int j = t + b * P;
#pragma unroll
          for (int r = 0; r < R; ++r) v[b * R + r] = xr(j + r * (L / R));
        }
        if constexpr (s < NS - 1) __syncthreads();
#pragma unroll
        for (int b = 0; b < E / R; ++b) {
          const int j = t + b * P;
          const int k = j % Ns;
#pragma unroll
          for (int r = 1; r < R; ++r) v[b * R + r] = c_mul(v[b * R + r], ld_tw(tw + two + (r - 1) * Ns + k));
          Dft<R, 1>::run(v + b * R);
        }
      });
    }
  }

  // visit the outputs of compute() in place: f(p, value&), p = frequency index
  template <class F>
  __device__ __forceinline__ static void for_outputs(int t, V (&v)[E], F&& f) {
    if constexpr (NS == 0) {
      f(t, v[0]);
    } else if constexpr (NS == 1) {
#pragma unroll
      for (int r = 0; r < E; ++r) f(r, v[r]);
    } else {
      constexpr int R = pl.radix[NS - 1];
      constexpr int Ns = plan_ns_before(pl, NS - 1);
#pragma unroll
      for (int b = 0; b < E / R; ++b)
#pragma unroll
        for (int r = 0; r < R; ++r) f(t + b * P + r * Ns, v[b * R + r]);
    }
  }

  // Reorder the outputs of compute() into stage-0 input order.  The last
  // stage leaves thread t with frequencies t + b*P + r*(L/R) (b < E/R, r < R)
  // in v[b*R + r]; since L/R = (E/R)*P these are exactly t + r'*P with
  // r' = b + r*(E/R), the elements stage 0 of a following transform of the
  // same line loads on this thread.  A compile-time register permutation:
  // a transform, a per-frequency multiply and an inverse transform need no
  // shared-memory round trip in between.
  __device__ __forceinline__ static void to_load_order(V (&v)[E]) {
    if constexpr (NS >= 2) {
      constexpr int R = pl.radix[NS - 1];
      V tmp[E];
#pragma unroll
      for (int b = 0; b < E / R; ++b)
#pragma unroll
        for (int r = 0; r < R; ++r) tmp[b + r * (E / R)] = v[b * R + r];
#pragma unroll
      for (int i = 0; i < E; ++i) v[i] = tmp[i];
    }
  }

  // hand the outputs of compute() to store(p, value), p = frequency index
  template <class Store>
  __device__ __forceinline__ static void emit(int t, V (&v)[E], Store&& store) {
    if constexpr (NS == 0) {
      store(t, v[0]);
    } else if constexpr (NS == 1) {
#pragma unroll
      for (int r = 0; r < E; ++r) store(r, v[r]);
    } else {
      constexpr int R = pl.radix[NS - 1];
      constexpr int Ns = plan_ns_before(pl, NS - 1);
#pragma unroll
      for (int b = 0; b < E / R; ++b) {
        const int j = t + b * P;
#pragma unroll
        for (int r = 0; r < R; ++r) store(j + r * Ns, v[b * R + r]);
      }
    }
  }

  // kSmemStore : the storer writes shared memory (barrier after the last
  //              stage's shared-memory reads).
  // kSyncAfterLoad : the loader reads shared memory (barrier before the first
  //              exchange overwrites it).
  template <bool kSmemStore, bool kSyncAfterLoad, class Load, class Store, class XW, class XR>
  __device__ __forceinline__ static void run(int t, const V* __restrict__ tw, Load&& load, Store&& store,
                                             XW&& xw, XR&& xr) {
    V v[E];
    compute(t, tw, load, xw, xr,
            [] {
              if constexpr (kSyncAfterLoad && NS >= 2) __syncthreads();
            },
            v);
    if constexpr (kSmemStore && NS >= 2) __syncthreads();
    emit(t, v, store);
  }
};

}  // namespace afg
