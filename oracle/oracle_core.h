/*
 * oracle_core.h - transform core of the oracle, instantiated by fft_oracle.c
 * for REAL = double (SFX = _d) and REAL = long double (SFX = _l).
 * TEST INFRASTRUCTURE ONLY (see fft_oracle.c).
 */

typedef struct {
  REAL re, im;
} SFX(cpx);

typedef struct {
  int n;
  int nf;
  int fac[ORC_MAX_FACTORS];
  SFX(cpx) * w;  /* w[k] = exp(-2*pi*i*k/n) */
  SFX(cpx) * tw; /* stage s (radix p, Ns = product of the earlier radices) at
                    tw + toff[s]: w_{Ns*p}^{q*k} at k*(p-1) + q-1, q in [1,p), k < Ns */
  long long toff[ORC_MAX_FACTORS];
} SFX(plan1d);

/* exp(-2*pi*i*m/d): integer octant reduction, then cos/sin on [0, pi/4] */
static void SFX(twid)(long long m, long long d, REAL* c, REAL* s) {
  m %= d;
  if (m < 0) m += d;
  long long o = (8 * m) / d, r = 8 * m - o * d;
  REAL phi = REAL_PI_4 * (REAL)r / (REAL)d, psi = REAL_PI_4 * (REAL)(d - r) / (REAL)d;
  REAL cc, ss;
  switch (o) {
    case 0: cc = TRIG_COS(phi); ss = TRIG_SIN(phi); break;
    case 1: cc = TRIG_SIN(psi); ss = TRIG_COS(psi); break;
    case 2: cc = -TRIG_SIN(phi); ss = TRIG_COS(phi); break;
    case 3: cc = -TRIG_COS(psi); ss = TRIG_SIN(psi); break;
    case 4: cc = -TRIG_COS(phi); ss = -TRIG_SIN(phi); break;
    case 5: cc = -TRIG_SIN(psi); ss = -TRIG_COS(psi); break;
    case 6: cc = TRIG_SIN(phi); ss = -TRIG_COS(phi); break;
    default: cc = TRIG_COS(psi); ss = -TRIG_SIN(psi); break;
  }
  *c = cc;
  *s = -ss;
}

static int SFX(plan_init)(SFX(plan1d) * p, int n) {
  p->n = n;
  p->nf = 0;
  int m = n;
  while (m % 4 == 0 && p->nf < ORC_MAX_FACTORS) { p->fac[p->nf++] = 4; m /= 4; }
  for (int f = 2; m > 1 && p->nf < ORC_MAX_FACTORS;) {
    if (m % f == 0) { p->fac[p->nf++] = f; m /= f; }
    else f = (f == 2) ? 3 : f + 2;
  }
  if (m != 1) return -1;
  long long ntw = 0, Ns = 1;
  for (int s = 0; s < p->nf; ++s) {
    p->toff[s] = ntw;
    ntw += Ns * (p->fac[s] - 1);
    Ns *= p->fac[s];
  }
  p->w = (SFX(cpx)*)malloc(sizeof(SFX(cpx)) * ((size_t)n + (size_t)ntw + 1));
  if (!p->w) return -1;
  p->tw = p->w + n;
  for (int k = 0; k < n; ++k) SFX(twid)(k, n, &p->w[k].re, &p->w[k].im);
  /* w_{Ns*p}^{q*k} = w_n^{q*k*(n/(Ns*p))}, the exponent below n */
  Ns = 1;
  for (int s = 0; s < p->nf; ++s) {
    const int r = p->fac[s];
    const long long step = n / (Ns * r);
    for (long long k = 0; k < Ns; ++k)
      for (int q = 1; q < r; ++q) p->tw[p->toff[s] + k * (r - 1) + q - 1] = p->w[q * k * step];
    Ns *= r;
  }
  return 0;
}

static void SFX(plan_free)(SFX(plan1d) * p) { free(p->w); }

static inline SFX(cpx) SFX(cmul)(SFX(cpx) a, SFX(cpx) b) {
  SFX(cpx) r;
  r.re = a.re * b.re - a.im * b.im;
  r.im = a.re * b.im + a.im * b.re;
  return r;
}

/* Stockham autosort, one stage per factor: stage s of radix p (Ns = product
 * of the earlier radices, m = n/p) takes x[j + q*m] for q < p, multiplies
 * entry q by w_{Ns*p}^{q*(j%Ns)}, runs the p-point DFT and writes output r at
 * (j/Ns)*Ns*p + j%Ns + r*Ns.  `in` is read by the first stage only; the
 * stages alternate between `out` and `tmp` so that the last one writes
 * `out` (both n entries). */
static void SFX(fft_line)(const SFX(plan1d) * P, const SFX(cpx) * in, SFX(cpx) * out, int sign, SFX(cpx) * tmp) {
  const int n = P->n, nf = P->nf;
  if (nf == 0) {
    out[0] = in[0];
    return;
  }
  const SFX(cpx)* src = in;
  long long Ns = 1;
  for (int s = 0; s < nf; ++s) {
    const int p = P->fac[s];
    const long long m = n / p;
    SFX(cpx)* dst = ((nf - 1 - s) % 2 == 0) ? out : tmp;
    const SFX(cpx)* t = P->tw + P->toff[s];
    for (long long j0 = 0; j0 < m; j0 += Ns) {
      for (long long k = 0; k < Ns; ++k) {
        const long long j = j0 + k;
        SFX(cpx) x[p];
        x[0] = src[j];
        for (int q = 1; q < p; ++q) {
          SFX(cpx) w = t[k * (p - 1) + q - 1];
          if (sign > 0) w.im = -w.im;
          x[q] = SFX(cmul)(src[j + q * m], w);
        }
        SFX(cpx)* y = dst + j0 * p + k;
        if (p == 2) {
          y[0].re = x[0].re + x[1].re; y[0].im = x[0].im + x[1].im;
          y[Ns].re = x[0].re - x[1].re; y[Ns].im = x[0].im - x[1].im;
        } else if (p == 4) {
          /* X[r] = sum_q x[q] w_4^{qr}; w_4 = -i (forward) or +i (backward) */
          const SFX(cpx) s02 = {x[0].re + x[2].re, x[0].im + x[2].im};
          const SFX(cpx) d02 = {x[0].re - x[2].re, x[0].im - x[2].im};
          const SFX(cpx) s13 = {x[1].re + x[3].re, x[1].im + x[3].im};
          const SFX(cpx) d13 = {x[1].re - x[3].re, x[1].im - x[3].im};
          SFX(cpx) rd; /* w_4 * d13 */
          if (sign < 0) { rd.re = d13.im; rd.im = -d13.re; }
          else { rd.re = -d13.im; rd.im = d13.re; }
          y[0].re = s02.re + s13.re; y[0].im = s02.im + s13.im;
          y[Ns].re = d02.re + rd.re; y[Ns].im = d02.im + rd.im;
          y[2 * Ns].re = s02.re - s13.re; y[2 * Ns].im = s02.im - s13.im;
          y[3 * Ns].re = d02.re - rd.re; y[3 * Ns].im = d02.im - rd.im;
        } else {
          /* direct p-point DFT: w_p^e = w_n^{(e mod p) * m} */
          for (int r = 0; r < p; ++r) {
            SFX(cpx) acc = x[0];
            for (int q = 1; q < p; ++q) {
              SFX(cpx) w = P->w[(long long)((q * r) % p) * m];
              if (sign > 0) w.im = -w.im;
              const SFX(cpx) v = SFX(cmul)(x[q], w);
              acc.re += v.re;
              acc.im += v.im;
            }
            y[r * Ns] = acc;
          }
        }
      }
    }
    src = dst;
    Ns *= p;
  }
}

static int SFX(fft1d)(int n, const double* in, double* out, int sign) {
  SFX(plan1d) p;
  if (n < 1 || SFX(plan_init)(&p, n)) return -1;
  SFX(cpx)* a = (SFX(cpx)*)malloc(sizeof(SFX(cpx)) * 3 * (size_t)n);
  for (int i = 0; i < n; ++i) { a[i].re = in[2 * i]; a[i].im = in[2 * i + 1]; }
  SFX(fft_line)(&p, a, a + n, sign, a + 2 * n);
  for (int i = 0; i < n; ++i) { out[2 * i] = (double)a[n + i].re; out[2 * i + 1] = (double)a[n + i].im; }
  free(a);
  SFX(plan_free)(&p);
  return 0;
}

/* ----------------------------------------------------------- line batches */
typedef struct {
  SFX(plan1d) pl;
  int L;          /* line length */
  int sign;
  /* complex axis pass */
  double* data;
  long long lstride, bstride, nb; /* line li: base = (li / nb)*bstride + (li % nb), element j at + j*lstride */
  /* real passes */
  const double* rin;
  double* rout;
  long long in_row, out_row; /* z passes */
  long long a, b;            /* strided real passes: [a][L][b] */
} SFX(batch);

/* Lines li of [b0, b1); on a strided axis up to ORC_COLS neighbouring
 * columns of one slab move together (each line position j is then one
 * contiguous run of the array), each transformed on its own as before. */
#define ORC_COLS 8
static void SFX(axis_worker)(void* ctx, long long b0, long long b1, int tid) {
  (void)tid;
  SFX(batch)* B = (SFX(batch)*)ctx;
  const int L = B->L;
  const int cols = B->lstride > 1 ? ORC_COLS : 1;
  SFX(cpx)* io = (SFX(cpx)*)malloc(sizeof(SFX(cpx)) * ((size_t)L * cols + 2 * (size_t)L + 8));
  SFX(cpx)* buf = io + (size_t)L * cols;
  for (long long li = b0; li < b1;) {
    const long long base = (li / B->nb) * B->bstride + (li % B->nb);
    long long c = B->nb - li % B->nb; /* columns left in this slab */
    if (c > cols) c = cols;
    if (c > b1 - li) c = b1 - li;
    for (int j = 0; j < L; ++j) {
      const double* s = B->data + 2 * (base + j * B->lstride);
      for (long long t = 0; t < c; ++t) {
        io[t * L + j].re = s[2 * t];
        io[t * L + j].im = s[2 * t + 1];
      }
    }
    for (long long t = 0; t < c; ++t) {
      SFX(fft_line)(&B->pl, io + t * L, buf, B->sign, buf + L);
      memcpy(io + t * L, buf, sizeof(SFX(cpx)) * (size_t)L);
    }
    for (int j = 0; j < L; ++j) {
      double* d = B->data + 2 * (base + j * B->lstride);
      for (long long t = 0; t < c; ++t) {
        d[2 * t] = (double)io[t * L + j].re;
        d[2 * t + 1] = (double)io[t * L + j].im;
      }
    }
    li += c;
  }
  free(io);
}

static int SFX(c2c_axis)(int n0, int n1, int w, int axis, double* data, int sign, int nthreads) {
  SFX(batch) B;
  memset(&B, 0, sizeof B);
  B.sign = sign;
  B.data = data;
  long long nlines;
  if (axis == 2) {
    B.L = w; B.lstride = 1; B.bstride = w; B.nb = 1; nlines = (long long)n0 * n1;
  } else if (axis == 1) {
    B.L = n1; B.lstride = w; B.bstride = (long long)n1 * w; B.nb = w; nlines = (long long)n0 * w;
  } else if (axis == 0) {
    B.L = n0; B.lstride = (long long)n1 * w; B.bstride = 0; B.nb = (long long)n1 * w; nlines = (long long)n1 * w;
  } else {
    return -1;
  }
  if (SFX(plan_init)(&B.pl, B.L)) return -1;
  orc_parallel(SFX(axis_worker), &B, nlines, nthreads);
  SFX(plan_free)(&B.pl);
  return 0;
}

/* r2c of one real line: full complex transform of (x, 0), keep k = 0..L/2 */
static void SFX(r2c_line)(SFX(batch) * B, SFX(cpx) * buf) {
  SFX(fft_line)(&B->pl, buf, buf + B->L, -1, buf + 2 * B->L);
}
/* c2r of one line from k = 0..L/2: Hermitian completion with the imaginary
 * parts of k = 0 and (even L) k = L/2 dropped, backward transform, real part */
static void SFX(c2r_line)(SFX(batch) * B, SFX(cpx) * buf) {
  const int L = B->L, H = L / 2 + 1;
  buf[0].im = 0;
  if (L % 2 == 0) buf[L / 2].im = 0;
  for (int k = H; k < L; ++k) {
    buf[k].re = buf[L - k].re;
    buf[k].im = -buf[L - k].im;
  }
  SFX(fft_line)(&B->pl, buf, buf + L, +1, buf + 2 * L);
}

/* Rows r and r+1 go through one complex transform of x_r + i x_{r+1}:
 * A[k] = (X[k] + conj X[L-k]) / 2, B[k] = (X[k] - conj X[L-k]) / 2i (both rows
 * are read before either is written, so in-place rows are fine); an odd last
 * row runs alone. */
static void SFX(r2c_z_worker)(void* ctx, long long b0, long long b1, int tid) {
  (void)tid;
  SFX(batch)* B = (SFX(batch)*)ctx;
  const int L = B->L, H = L / 2 + 1;
  SFX(cpx)* buf = (SFX(cpx)*)malloc(sizeof(SFX(cpx)) * (3 * (size_t)L + 8));
  long long r = b0;
  for (; r + 1 < b1; r += 2) {
    const double* s0 = B->rin + r * B->in_row;
    const double* s1 = s0 + B->in_row;
    for (int j = 0; j < L; ++j) { buf[j].re = s0[j]; buf[j].im = s1[j]; }
    SFX(fft_line)(&B->pl, buf, buf + L, -1, buf + 2 * L);
    const SFX(cpx)* X = buf + L;
    double* d0 = B->rout + 2 * r * B->out_row;
    double* d1 = d0 + 2 * B->out_row;
    for (int k = 0; k < H; ++k) {
      const SFX(cpx) x = X[k], y = X[k == 0 ? 0 : L - k];
      d0[2 * k] = (double)((REAL)0.5 * (x.re + y.re));
      d0[2 * k + 1] = (double)((REAL)0.5 * (x.im - y.im));
      d1[2 * k] = (double)((REAL)0.5 * (x.im + y.im));
      d1[2 * k + 1] = (double)((REAL)-0.5 * (x.re - y.re));
    }
  }
  for (; r < b1; ++r) {
    const double* s = B->rin + r * B->in_row;
    for (int j = 0; j < L; ++j) { buf[j].re = s[j]; buf[j].im = 0; }
    SFX(r2c_line)(B, buf);
    double* d = B->rout + 2 * r * B->out_row;
    for (int k = 0; k < H; ++k) { d[2 * k] = (double)buf[L + k].re; d[2 * k + 1] = (double)buf[L + k].im; }
  }
  free(buf);
}

/* Rows r and r+1 go through one backward transform of A + iB (A, B their
 * Hermitian completions, imaginary parts of k = 0 and L/2 dropped): the
 * result is a + ib, a and b the two real rows; an odd last row runs alone. */
static void SFX(c2r_z_worker)(void* ctx, long long b0, long long b1, int tid) {
  (void)tid;
  SFX(batch)* B = (SFX(batch)*)ctx;
  const int L = B->L, H = L / 2 + 1;
  SFX(cpx)* buf = (SFX(cpx)*)malloc(sizeof(SFX(cpx)) * (3 * (size_t)L + 8));
  long long r = b0;
  for (; r + 1 < b1; r += 2) {
    const double* h0 = B->rin + 2 * r * B->in_row;
    const double* h1 = h0 + 2 * B->in_row;
    for (int p = 0; p < L; ++p) {
      const int q = p < H ? p : L - p;
      REAL ar = h0[2 * q], ai = h0[2 * q + 1], br = h1[2 * q], bi = h1[2 * q + 1];
      if (p == 0 || 2 * p == L) ai = bi = 0;
      if (p >= H) { ai = -ai; bi = -bi; }
      buf[p].re = ar - bi;
      buf[p].im = ai + br;
    }
    SFX(fft_line)(&B->pl, buf, buf + L, +1, buf + 2 * L);
    double* d0 = B->rout + r * B->out_row;
    double* d1 = d0 + B->out_row;
    for (int j = 0; j < L; ++j) { d0[j] = (double)buf[L + j].re; d1[j] = (double)buf[L + j].im; }
  }
  for (; r < b1; ++r) {
    const double* s = B->rin + 2 * r * B->in_row;
    for (int k = 0; k < H; ++k) { buf[k].re = s[2 * k]; buf[k].im = s[2 * k + 1]; }
    SFX(c2r_line)(B, buf);
    double* d = B->rout + r * B->out_row;
    for (int j = 0; j < L; ++j) d[j] = (double)buf[L + j].re;
  }
  free(buf);
}

static int SFX(r2c_z)(long long rows, int n2, const double* in, long long in_row, double* out, long long out_row,
                      int nthreads) {
  SFX(batch) B;
  memset(&B, 0, sizeof B);
  B.L = n2; B.rin = in; B.rout = out; B.in_row = in_row; B.out_row = out_row;
  if (SFX(plan_init)(&B.pl, n2)) return -1;
  orc_parallel(SFX(r2c_z_worker), &B, rows, nthreads);
  SFX(plan_free)(&B.pl);
  return 0;
}

static int SFX(c2r_z)(long long rows, int n2, const double* in, long long in_row, double* out, long long out_row,
                      int nthreads) {
  SFX(batch) B;
  memset(&B, 0, sizeof B);
  B.L = n2; B.rin = in; B.rout = out; B.in_row = in_row; B.out_row = out_row;
  if (SFX(plan_init)(&B.pl, n2)) return -1;
  orc_parallel(SFX(c2r_z_worker), &B, rows, nthreads);
  SFX(plan_free)(&B.pl);
  return 0;
}

static void SFX(r2c_s_worker)(void* ctx, long long b0, long long b1, int tid) {
  (void)tid;
  SFX(batch)* B = (SFX(batch)*)ctx;
  const int L = B->L, H = L / 2 + 1;
  SFX(cpx)* buf = (SFX(cpx)*)malloc(sizeof(SFX(cpx)) * (3 * (size_t)L + 8));
  for (long long li = b0; li < b1; ++li) {
    long long ai = li / B->b, bi = li % B->b;
    const double* s = B->rin + ai * L * B->b + bi;
    for (int j = 0; j < L; ++j) { buf[j].re = s[j * B->b]; buf[j].im = 0; }
    SFX(r2c_line)(B, buf);
    double* d = B->rout + 2 * (ai * H * B->b + bi);
    for (int k = 0; k < H; ++k) {
      d[2 * k * B->b] = (double)buf[L + k].re;
      d[2 * k * B->b + 1] = (double)buf[L + k].im;
    }
  }
  free(buf);
}

static void SFX(c2r_s_worker)(void* ctx, long long b0, long long b1, int tid) {
  (void)tid;
  SFX(batch)* B = (SFX(batch)*)ctx;
  const int L = B->L, H = L / 2 + 1;
  SFX(cpx)* buf = (SFX(cpx)*)malloc(sizeof(SFX(cpx)) * (3 * (size_t)L + 8));
  for (long long li = b0; li < b1; ++li) {
    long long ai = li / B->b, bi = li % B->b;
    const double* s = B->rin + 2 * (ai * H * B->b + bi);
    for (int k = 0; k < H; ++k) { buf[k].re = s[2 * k * B->b]; buf[k].im = s[2 * k * B->b + 1]; }
    SFX(c2r_line)(B, buf);
    double* d = B->rout + ai * L * B->b + bi;
    for (int j = 0; j < L; ++j) d[j * B->b] = (double)buf[L + j].re;
  }
  free(buf);
}

static int SFX(r2c_strided)(long long a, int L, long long b, const double* in, double* out, int nthreads) {
  SFX(batch) B;
  memset(&B, 0, sizeof B);
  B.L = L; B.a = a; B.b = b; B.rin = in; B.rout = out;
  if (SFX(plan_init)(&B.pl, L)) return -1;
  orc_parallel(SFX(r2c_s_worker), &B, a * b, nthreads);
  SFX(plan_free)(&B.pl);
  return 0;
}

static int SFX(c2r_strided)(long long a, int L, long long b, const double* in, double* out, int nthreads) {
  SFX(batch) B;
  memset(&B, 0, sizeof B);
  B.L = L; B.a = a; B.b = b; B.rin = in; B.rout = out;
  if (SFX(plan_init)(&B.pl, L)) return -1;
  orc_parallel(SFX(c2r_s_worker), &B, a * b, nthreads);
  SFX(plan_free)(&B.pl);
  return 0;
}
