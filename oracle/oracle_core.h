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
 * (j/Ns)*Ns*p + j%Ns + r*Ns.  V lines run together, element-major (entry j of
 * line t at x[j*V + t]), sharing each twiddle.  `in` is read by the first
 * stage only; the stages alternate between `out` and `tmp` so that the last
 * one writes `out` (both n*V entries). */
static void SFX(fft_lines)(const SFX(plan1d) * P, const SFX(cpx) * in, SFX(cpx) * out, int sign, SFX(cpx) * tmp,
                           int V) {
  const int n = P->n, nf = P->nf;
  if (nf == 0) {
    for (int t = 0; t < V; ++t) out[t] = in[t];
    return;
  }
  const REAL sg = sign < 0 ? (REAL)1 : (REAL)-1; /* w_4 * d = (sg * d.im, -sg * d.re) */
  const SFX(cpx)* src = in;
  long long Ns = 1;
  for (int s = 0; s < nf; ++s) {
    const int p = P->fac[s];
    const long long m = n / p, xs = m * V;
    SFX(cpx)* dst = ((nf - 1 - s) % 2 == 0) ? out : tmp;
    const SFX(cpx)* tw = P->tw + P->toff[s];
    const long long ys = Ns * V;
    for (long long j0 = 0; j0 < m; j0 += Ns) {
      for (long long k = 0; k < Ns; ++k) {
        const SFX(cpx)* x = src + (j0 + k) * V;
        SFX(cpx)* y = dst + (j0 * p + k) * V;
        if (p == 2) {
          SFX(cpx) w = tw[k];
          if (sign > 0) w.im = -w.im;
          for (int t = 0; t < V; ++t) {
            const SFX(cpx) a = x[t], b = SFX(cmul)(x[xs + t], w);
            y[t].re = a.re + b.re; y[t].im = a.im + b.im;
            y[ys + t].re = a.re - b.re; y[ys + t].im = a.im - b.im;
          }
        } else if (p == 4) {
          /* X[r] = sum_q x[q] w_4^{qr}; w_4 = -i (forward) or +i (backward) */
          SFX(cpx) w1 = tw[3 * k], w2 = tw[3 * k + 1], w3 = tw[3 * k + 2];
          if (sign > 0) { w1.im = -w1.im; w2.im = -w2.im; w3.im = -w3.im; }
          for (int t = 0; t < V; ++t) {
            const SFX(cpx) a0 = x[t], a1 = SFX(cmul)(x[xs + t], w1), a2 = SFX(cmul)(x[2 * xs + t], w2),
                           a3 = SFX(cmul)(x[3 * xs + t], w3);
            const SFX(cpx) s02 = {a0.re + a2.re, a0.im + a2.im};
            const SFX(cpx) d02 = {a0.re - a2.re, a0.im - a2.im};
            const SFX(cpx) s13 = {a1.re + a3.re, a1.im + a3.im};
            const SFX(cpx) d13 = {a1.re - a3.re, a1.im - a3.im};
            const SFX(cpx) rd = {sg * d13.im, -sg * d13.re};
            y[t].re = s02.re + s13.re; y[t].im = s02.im + s13.im;
            y[ys + t].re = d02.re + rd.re; y[ys + t].im = d02.im + rd.im;
            y[2 * ys + t].re = s02.re - s13.re; y[2 * ys + t].im = s02.im - s13.im;
            y[3 * ys + t].re = d02.re - rd.re; y[3 * ys + t].im = d02.im - rd.im;
          }
        } else {
          /* direct p-point DFT: w_p^e = w_n^{(e mod p) * m} */
          SFX(cpx) xq[p];
          for (int t = 0; t < V; ++t) {
            xq[0] = x[t];
            for (int q = 1; q < p; ++q) {
              SFX(cpx) w = tw[k * (p - 1) + q - 1];
              if (sign > 0) w.im = -w.im;
              xq[q] = SFX(cmul)(x[q * xs + t], w);
            }
            for (int r = 0; r < p; ++r) {
              SFX(cpx) acc = xq[0];
              for (int q = 1; q < p; ++q) {
                SFX(cpx) w = P->w[(long long)((q * r) % p) * m];
                if (sign > 0) w.im = -w.im;
                const SFX(cpx) v = SFX(cmul)(xq[q], w);
                acc.re += v.re;
                acc.im += v.im;
              }
              y[r * ys + t] = acc;
            }
          }
        }
      }
    }
    src = dst;
    Ns *= p;
  }
}

/* one line (V = 1) */
static void SFX(fft_line)(const SFX(plan1d) * P, const SFX(cpx) * in, SFX(cpx) * out, int sign, SFX(cpx) * tmp) {
  SFX(fft_lines)(P, in, out, sign, tmp, 1);
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

/* Lines li of [b0, b1), ORC_COLS at a time through fft_lines: on a strided
 * axis neighbouring columns of one slab (each line position j is one
 * contiguous run of the array), on the contiguous axis consecutive rows. */
#define ORC_COLS 8
static void SFX(axis_worker)(void* ctx, long long b0, long long b1, int tid) {
  (void)tid;
  SFX(batch)* B = (SFX(batch)*)ctx;
  const int L = B->L;
  const size_t blk = (size_t)L * ORC_COLS;
  SFX(cpx)* io = (SFX(cpx)*)malloc(sizeof(SFX(cpx)) * (3 * blk + 8));
  SFX(cpx)* res = io + blk;
  long long base[ORC_COLS];
  for (long long li = b0; li < b1;) {
    long long c = B->nb > 1 ? B->nb - li % B->nb : ORC_COLS; /* lines left in this slab */
    if (c > ORC_COLS) c = ORC_COLS;
    if (c > b1 - li) c = b1 - li;
    for (long long t = 0; t < c; ++t) base[t] = ((li + t) / B->nb) * B->bstride + (li + t) % B->nb;
    if (B->lstride > 1) { /* strided: row j of the block is one run of c entries */
      for (int j = 0; j < L; ++j) {
        const double* s = B->data + 2 * (base[0] + j * B->lstride);
        for (long long t = 0; t < c; ++t) { io[j * c + t].re = s[2 * t]; io[j * c + t].im = s[2 * t + 1]; }
      }
    } else {
      for (long long t = 0; t < c; ++t) {
        const double* s = B->data + 2 * base[t];
        for (int j = 0; j < L; ++j) { io[j * c + t].re = s[2 * j]; io[j * c + t].im = s[2 * j + 1]; }
      }
    }
    SFX(fft_lines)(&B->pl, io, res, B->sign, res + blk, (int)c);
    if (B->lstride > 1) {
      for (int j = 0; j < L; ++j) {
        double* d = B->data + 2 * (base[0] + j * B->lstride);
        for (long long t = 0; t < c; ++t) { d[2 * t] = (double)res[j * c + t].re; d[2 * t + 1] = (double)res[j * c + t].im; }
      }
    } else {
      for (long long t = 0; t < c; ++t) {
        double* d = B->data + 2 * base[t];
        for (int j = 0; j < L; ++j) { d[2 * j] = (double)res[j * c + t].re; d[2 * j + 1] = (double)res[j * c + t].im; }
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
 * A[k] = (X[k] + conj X[L-k]) / 2, B[k] = (X[k] - conj X[L-k]) / 2i; up to
 * ORC_COLS such pairs run together through fft_lines.  Every row of a block
 * is read before any is written, so in-place rows are fine; an odd last row
 * pairs with zeros. */
static void SFX(r2c_z_worker)(void* ctx, long long b0, long long b1, int tid) {
  (void)tid;
  SFX(batch)* B = (SFX(batch)*)ctx;
  const int L = B->L, H = L / 2 + 1;
  const size_t blk = (size_t)L * ORC_COLS;
  SFX(cpx)* io = (SFX(cpx)*)malloc(sizeof(SFX(cpx)) * (3 * blk + 8));
  SFX(cpx)* X = io + blk;
  for (long long r = b0; r < b1;) {
    long long rows = b1 - r;
    if (rows > 2 * ORC_COLS) rows = 2 * ORC_COLS;
    const int c = (int)((rows + 1) / 2);
    for (int t = 0; t < c; ++t) {
      const double* s0 = B->rin + (r + 2 * t) * B->in_row;
      const int two = 2 * t + 1 < rows;
      for (int j = 0; j < L; ++j) {
        io[j * c + t].re = s0[j];
        io[j * c + t].im = two ? s0[B->in_row + j] : 0;
      }
    }
    SFX(fft_lines)(&B->pl, io, X, -1, X + blk, c);
    for (int t = 0; t < c; ++t) {
      double* d0 = B->rout + 2 * (r + 2 * t) * B->out_row;
      const int two = 2 * t + 1 < rows;
      for (int k = 0; k < H; ++k) {
        const SFX(cpx) x = X[k * c + t], y = X[(k == 0 ? 0 : L - k) * c + t];
        d0[2 * k] = (double)((REAL)0.5 * (x.re + y.re));
        d0[2 * k + 1] = (double)((REAL)0.5 * (x.im - y.im));
        if (two) {
          d0[2 * B->out_row + 2 * k] = (double)((REAL)0.5 * (x.im + y.im));
          d0[2 * B->out_row + 2 * k + 1] = (double)((REAL)-0.5 * (x.re - y.re));
        }
      }
    }
    r += rows;
  }
  free(io);
}

/* Rows r and r+1 go through one backward transform of A + iB (A, B their
 * Hermitian completions, imaginary parts of k = 0 and L/2 dropped): the
 * result is a + ib, a and b the two real rows; up to ORC_COLS pairs run
 * together, an odd last row pairs with zeros. */
static void SFX(c2r_z_worker)(void* ctx, long long b0, long long b1, int tid) {
  (void)tid;
  SFX(batch)* B = (SFX(batch)*)ctx;
  const int L = B->L, H = L / 2 + 1;
  const size_t blk = (size_t)L * ORC_COLS;
  SFX(cpx)* io = (SFX(cpx)*)malloc(sizeof(SFX(cpx)) * (3 * blk + 8));
  SFX(cpx)* Y = io + blk;
  for (long long r = b0; r < b1;) {
    long long rows = b1 - r;
    if (rows > 2 * ORC_COLS) rows = 2 * ORC_COLS;
    const int c = (int)((rows + 1) / 2);
    for (int t = 0; t < c; ++t) {
      const int two = 2 * t + 1 < rows;
      const double* h0 = B->rin + 2 * (r + 2 * t) * B->in_row;
      const double* h1 = two ? h0 + 2 * B->in_row : h0;
      for (int p = 0; p < L; ++p) {
        const int q = p < H ? p : L - p;
        REAL ar = h0[2 * q], ai = h0[2 * q + 1], br = 0, bi = 0;
        if (two) { br = h1[2 * q]; bi = h1[2 * q + 1]; }
        if (p == 0 || 2 * p == L) ai = bi = 0;
        if (p >= H) { ai = -ai; bi = -bi; }
        io[p * c + t].re = ar - bi;
        io[p * c + t].im = ai + br;
      }
    }
    SFX(fft_lines)(&B->pl, io, Y, +1, Y + blk, c);
    for (int t = 0; t < c; ++t) {
      double* d0 = B->rout + (r + 2 * t) * B->out_row;
      const int two = 2 * t + 1 < rows;
      for (int j = 0; j < L; ++j) {
        d0[j] = (double)Y[j * c + t].re;
        if (two) d0[B->out_row + j] = (double)Y[j * c + t].im;
      }
    }
    r += rows;
  }
  free(io);
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
