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
  SFX(cpx) * w; /* w[k] = exp(-2*pi*i*k/n) */
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
  p->w = (SFX(cpx)*)malloc(sizeof(SFX(cpx)) * (size_t)n);
  if (!p->w) return -1;
  for (int k = 0; k < n; ++k) SFX(twid)(k, n, &p->w[k].re, &p->w[k].im);
  return 0;
}

static void SFX(plan_free)(SFX(plan1d) * p) { free(p->w); }

static inline SFX(cpx) SFX(cmul)(SFX(cpx) a, SFX(cpx) b) {
  SFX(cpx) r;
  r.re = a.re * b.re - a.im * b.im;
  r.im = a.re * b.im + a.im * b.re;
  return r;
}

/* w_N^e for the transform sign (conjugate table entry for sign > 0) */
static inline SFX(cpx) SFX(wexp)(const SFX(cpx) * w, long long N, long long e, int sign) {
  SFX(cpx) t = w[e % N];
  if (sign > 0) t.im = -t.im;
  return t;
}
/* the same for 0 <= e < N (no reduction) */
static inline SFX(cpx) SFX(wexp_in)(const SFX(cpx) * w, long long e, int sign) {
  SFX(cpx) t = w[e];
  if (sign > 0) t.im = -t.im;
  return t;
}

/* Recursive decimation in time.  Sub-transform of length n reads in[j*is]
 * for j < n; w is the table of the top-level length N and wstep = N/n.
 * The twiddle exponent q*k*wstep stays below p*m*wstep = N.  A last factor
 * (m == 1) reads its inputs directly: its length-1 sub-transforms are
 * copies and its twiddles are w^0 = 1. */
static void SFX(rec)(const SFX(cpx) * in, long long is, SFX(cpx) * out, int n, const int* fac, const SFX(cpx) * w,
                     long long N, long long wstep, int sign, SFX(cpx) * tmp) {
  if (n == 1) {
    out[0] = in[0];
    return;
  }
  const int p = fac[0], m = n / p;
  if (m > 1)
    for (int q = 0; q < p; ++q) SFX(rec)(in + q * is, is * p, out + q * m, m, fac + 1, w, N, wstep * p, sign, tmp);
  for (int k = 0; k < m; ++k) {
    if (m == 1)
      for (int q = 0; q < p; ++q) tmp[q] = in[q * is];
    else
      for (int q = 0; q < p; ++q) tmp[q] = SFX(cmul)(out[q * m + k], SFX(wexp_in)(w, (long long)q * k * wstep, sign));
    if (p == 2) {
      SFX(cpx) a = tmp[0], b = tmp[1];
      out[k].re = a.re + b.re; out[k].im = a.im + b.im;
      out[m + k].re = a.re - b.re; out[m + k].im = a.im - b.im;
    } else if (p == 4) {
      /* X[r] = sum_q t[q] w_4^{qr}; w_4 = -i (forward) or +i (backward) */
      SFX(cpx) s02 = {tmp[0].re + tmp[2].re, tmp[0].im + tmp[2].im};
      SFX(cpx) d02 = {tmp[0].re - tmp[2].re, tmp[0].im - tmp[2].im};
      SFX(cpx) s13 = {tmp[1].re + tmp[3].re, tmp[1].im + tmp[3].im};
      SFX(cpx) d13 = {tmp[1].re - tmp[3].re, tmp[1].im - tmp[3].im};
      SFX(cpx) rd; /* w_4 * d13 */
      if (sign < 0) { rd.re = d13.im; rd.im = -d13.re; }
      else { rd.re = -d13.im; rd.im = d13.re; }
      out[k].re = s02.re + s13.re; out[k].im = s02.im + s13.im;
      out[m + k].re = d02.re + rd.re; out[m + k].im = d02.im + rd.im;
      out[2 * m + k].re = s02.re - s13.re; out[2 * m + k].im = s02.im - s13.im;
      out[3 * m + k].re = d02.re - rd.re; out[3 * m + k].im = d02.im - rd.im;
    } else {
      for (int r = 0; r < p; ++r) {
        SFX(cpx) acc = {0, 0};
        for (int q = 0; q < p; ++q) {
          SFX(cpx) t = SFX(cmul)(tmp[q], SFX(wexp)(w, N, (long long)q * r * m * wstep, sign));
          acc.re += t.re;
          acc.im += t.im;
        }
        out[r * m + k] = acc;
      }
    }
  }
}

static void SFX(fft_line)(const SFX(plan1d) * p, const SFX(cpx) * in, SFX(cpx) * out, int sign, SFX(cpx) * tmp) {
  SFX(rec)(in, 1, out, p->n, p->fac, p->w, p->n, 1, sign, tmp);
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
