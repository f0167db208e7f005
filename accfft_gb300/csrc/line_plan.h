// Radix plans shared by the device line engine (compile time) and the host
// plan layer (twiddle tables at plan time).  Plain C++17: no CUDA types.
#pragma once
#if defined(__CUDACC__)
#define AFG_HD __host__ __device__
#else
#define AFG_HD
#endif

namespace afg {

// --------------------------------------------------------------- line plans
// A plan splits L = E * P: stage 0 has radix E, later radices all divide E so
// every thread owns exactly E/R butterflies in every stage.  Among all E <= 32
// the plan with the fewest stages wins (each stage is one shared-memory
// exchange); ties prefer P >= pmin threads per line (coalesced loads on
// contiguous lines) and E near the preferred register footprint.
struct LinePlan {
  int L, E, P, ns;
  int radix[16];
};

// greedy factorisation of L/E into divisors of E (largest first); returns the
// number of stages, 0 if impossible
AFG_HD constexpr int plan_greedy(int L, int E, int* rad) {
  int rem = L / E, ns = 1;
  rad[0] = E;
  while (rem > 1) {
    int d = 0;
    for (int c = E; c >= 2; --c)
      if (E % c == 0 && rem % c == 0) { d = c; break; }
    if (d == 0 || ns >= 16) return 0;
    rad[ns++] = d; rem /= d;
  }
  return ns;
}

AFG_HD constexpr LinePlan plan_for(int L, bool dbl, int emax = 32) {
  LinePlan pl{};
  pl.L = L; pl.E = 0; pl.P = 0; pl.ns = 0;
  for (int i = 0; i < 16; ++i) pl.radix[i] = 1;
  if (L == 1) { pl.E = 1; pl.P = 1; return pl; }
  const int epref = dbl ? (L >= 256 ? 16 : 8) : (L >= 512 ? 32 : 16);
  const int pmin = dbl ? 2 : 4;
  long best = -1;
  for (int E = 2; E <= emax && E <= L; ++E) {
    if (L % E) continue;
    int rad[16] = {};
    int ns = plan_greedy(L, E, rad);
    if (ns == 0) continue;
    int P = L / E;
    long cost = 100L * ns + ((P < pmin && L >= 2 * pmin) ? 50 : 0) + (E > epref ? 30 : 0) + (E > epref ? E - epref : epref - E);
    if (best < 0 || cost < best) {
      best = cost;
      pl.E = E; pl.P = P; pl.ns = ns;
      for (int i = 0; i < 16; ++i) pl.radix[i] = i < ns ? rad[i] : 1;
    }
  }
  return pl;   // E == 0 marks "no plan" (a prime factor above 32)
}

// plan with a fixed first radix E (E must divide L); E == 0 marks failure
AFG_HD constexpr LinePlan plan_with_e(int L, int E) {
  LinePlan pl{};
  pl.L = L; pl.E = 0; pl.P = 0; pl.ns = 0;
  for (int i = 0; i < 16; ++i) pl.radix[i] = 1;
  if (L == 1) { pl.E = 1; pl.P = 1; return pl; }
  if (E < 2 || L % E) return pl;
  int rad[16] = {};
  int ns = plan_greedy(L, E, rad);
  if (ns == 0) return pl;
  pl.E = E; pl.P = L / E; pl.ns = ns;
  for (int i = 0; i < 16; ++i) pl.radix[i] = i < ns ? rad[i] : 1;
  return pl;
}

// Double-float lines hold a complex value in four floats and need many
// temporaries per add, so they keep E <= 8 where the length allows: more
// warps per SM hide the dependent add chains (measured 2.9x faster than
// E = 32 for 512-point strided lines).  Lengths with no such plan fall back
// to the double plan.
AFG_HD constexpr LinePlan plan_for_df(int L) {
  LinePlan pl = plan_for(L, true, 8);
  return pl.E ? pl : plan_for(L, true);
}

// plan class: 0 float, 1 double, 2 double-float
AFG_HD constexpr LinePlan plan_select(int L, int cls, int E) {
  return E ? plan_with_e(L, E) : (cls == 2 ? plan_for_df(L) : plan_for(L, cls == 1));
}

// product of the radices of stages [0, s)
AFG_HD constexpr int plan_ns_before(const LinePlan& pl, int s) {
  int n = 1;
  for (int i = 0; i < s; ++i) n *= pl.radix[i];
  return n;
}
// offset of stage s in the stage-twiddle table; stage s >= 1 stores
// w_{Ns*R}^{k*r} at (r-1)*Ns + k for r in [1,R), k in [0,Ns)
AFG_HD constexpr int plan_tw_offset(const LinePlan& pl, int s) {
  int o = 0;
  for (int i = 1; i < s; ++i) o += (pl.radix[i] - 1) * plan_ns_before(pl, i);
  return o;
}
AFG_HD constexpr int plan_tw_size(const LinePlan& pl) { return plan_tw_offset(pl, pl.ns); }

}  // namespace afg
