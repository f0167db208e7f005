// Tensor-core line engine (float): the radix-16 stages of a Stockham line FFT
// as small dense matrix products on the 5th-generation tensor cores.
//
// A radix-16 stage applies the 16-point DFT matrix W to one butterfly per
// thread.  Written in real arithmetic, y = W x is a 32x32 real matrix
//     [Yr]   [ Wr  -Wi ] [Xr]
//     [Yi] = [ Wi   Wr ] [Xi]
// times a 32-vector.  The CTA's butterflies form the rows of A (M = 128 rows
// per block, one row per thread: K = 32 reals of its butterfly), B = W^T
// (N = 32 rows, K = 32) is the DFT matrix, and D = A B^T lands in tensor
// memory with row i = thread i's 32 outputs, so tcgen05.ld returns each
// thread exactly its own butterfly's outputs and the Stockham data flow of
// LineFFT is unchanged.
//
// Precision forms (FP32 accumulation in both):
//   TcForm::TF32x3  x = hi + lo, hi = tf32(x), lo = tf32(x - hi), for the
//                   data and the DFT matrix; D = A_lo B_hi + A_hi B_lo +
//                   A_hi B_hi (kind::tf32, K = 8 per MMA)
//   TcForm::BF16x6  x = hi + mid + lo, three bf16 parts (24 bits: exact for
//                   float data, DFT matrix split from the double value);
//                   D = the six products down to relative order 2^-16
//                   (A_lo B_hi + A_mid B_mid + A_hi B_lo, A_mid B_hi + A_hi
//                   B_mid, A_hi B_hi; smallest first), FP32-class accuracy
//                   (kind::f16 with bf16 operands, K = 16 per MMA)
//
// Operands: A in tensor memory, written by each thread from its registers
// with tcgen05.st (row i of a 128-row block = lane i, one part per 32
// columns: bf16 pairs or tf32 values along K), so the data never passes
// through shared memory on its way to the tensor core.  B (= W^T, 32 x 32,
// one matrix per part) sits in shared memory in the canonical K-major layout
// without swizzle: 8-row x 16-byte core matrices, adjacent along K at LBO =
// 128 B, adjacent 8-row groups at SBO = (row bytes / 16) * 128 B.  Each
// 128-row block owns 128 tensor-memory columns: the A parts at 0, 32 (and
// 64), D at 96.
//
// Every wait on the MMA-completion mbarrier is bounded (TcCtx::limit polls,
// by lane 0 of each warp).  A wait that gives up sets the error word, then
// drains: it waits again, up to kTcDrainPolls, for the products already
// issued, so no MMA still writes tensor memory when the kernel frees it.
// After that the engine issues and waits no more, and the kernel always
// reaches its end.
#pragma once
#include <cstdint>
#include "fft_core.cuh"

namespace afg {

enum class TcForm : int { TF32x3 = 1, BF16x6 = 2 };

template <TcForm F> struct TcTraits;
template <> struct TcTraits<TcForm::TF32x3> {
  static constexpr int parts = 2;           // hi, lo
  static constexpr int row_bytes = 128;     // a B row: 32 tf32
  static constexpr int kstep = 8;           // K per MMA
  static constexpr uint32_t fmt = 2;        // TF32 in the A/B format fields
  static constexpr int nprod = 3;
  // products (A part, B part), smallest first
  __host__ __device__ static constexpr int pa(int i) { return i == 0 ? 1 : 0; }
  __host__ __device__ static constexpr int pb(int i) { return i == 1 ? 1 : 0; }
};
template <> struct TcTraits<TcForm::BF16x6> {
  static constexpr int parts = 3;           // hi, mid, lo
  static constexpr int row_bytes = 64;      // a B row: 32 bf16
  static constexpr int kstep = 16;
  static constexpr uint32_t fmt = 1;        // BF16
  static constexpr int nprod = 6;
  __host__ __device__ static constexpr int pa(int i) { return i == 0 ? 2 : i == 1 ? 1 : i == 2 ? 0 : i == 3 ? 1 : 0; }
  __host__ __device__ static constexpr int pb(int i) { return i == 0 ? 0 : i == 1 ? 1 : i == 2 ? 2 : i == 3 ? 0 : i == 4 ? 1 : 0; }
};

// tensor-memory columns of one 128-row block: A part q at 32 q, D at 96
constexpr int kTcBlockCols = 128;
constexpr int kTcDCol = 96;

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// 64-bit shared-memory matrix descriptor: start >> 4 in [0,14), LBO >> 4 in
// [16,30), SBO >> 4 in [32,46), the fixed value 1 at bit 46, base offset 0,
// relative LBO, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((addr & 0x3FFFFu) >> 4);
  d |= static_cast<uint64_t>((lbo & 0x3FFFFu) >> 4) << 16;
  d |= static_cast<uint64_t>((sbo & 0x3FFFFu) >> 4) << 32;
  d |= static_cast<uint64_t>(1) << 46;
  return d;
}

// 32-bit instruction descriptor: D format F32 (bits 4-5 = 1), A and B formats
// (bits 7-9, 10-12), both K-major (bits 15, 16 = 0), N >> 3 at bit 17,
// M >> 4 at bit 24
template <TcForm F>
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
  return (1u << 4) | (TcTraits<F>::fmt << 7) | (TcTraits<F>::fmt << 10) |
         (static_cast<uint32_t>(N >> 3) << 17) | (static_cast<uint32_t>(M >> 4) << 24);
}

__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// D (tensor memory) += A (tensor memory) * B (shared-memory descriptor)
template <TcForm F>
__device__ __forceinline__ void mma_tmem_a(uint32_t d_tmem, uint32_t a_tmem, uint64_t bdesc, uint32_t idesc,
                                           uint32_t accumulate) {
  if constexpr (F == TcForm::TF32x3) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
        "r"(a_tmem), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
  } else {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
        "r"(a_tmem), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
  }
}

__device__ __forceinline__ bool mbar_try(uint32_t mbar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(mbar), "r"(parity)
      : "memory");
  return done != 0;
}

// this warp's 32 lanes x 16 / 32 consecutive columns from registers
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
          taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
      "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
      : "memory");
}
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
      "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
      "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(r[16]), "r"(r[17]), "r"(r[18]),
      "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]), "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]),
      "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31])
      : "memory");
}

// cos(2 pi m / 16), m = 0..15, evaluated by the compiler (sin(2 pi m / 16) =
// cos(2 pi (m - 4) / 16)); the device reads them, it never evaluates them
__constant__ double kTcCos16[16] = {
    ce_trig2pi(0, 16, false),  ce_trig2pi(1, 16, false),  ce_trig2pi(2, 16, false),  ce_trig2pi(3, 16, false),
    ce_trig2pi(4, 16, false),  ce_trig2pi(5, 16, false),  ce_trig2pi(6, 16, false),  ce_trig2pi(7, 16, false),
    ce_trig2pi(8, 16, false),  ce_trig2pi(9, 16, false),  ce_trig2pi(10, 16, false), ce_trig2pi(11, 16, false),
    ce_trig2pi(12, 16, false), ce_trig2pi(13, 16, false), ce_trig2pi(14, 16, false), ce_trig2pi(15, 16, false)};

// ----------------------------------------------------------- per-CTA context
// Shared-memory state of the engine; tc_begin() sets it up, tc_end() frees
// the tensor memory.
struct TcCtx {
  unsigned char* b;      // parts x 32 x row_bytes: the parts of W^T
  uint64_t* mbar;        // MMA completion
  uint32_t* tmem_slot;   // tensor-memory base address written by tcgen05.alloc
  uint32_t tmem;
  uint32_t phase;
  bool dead;             // a wait gave up: issue and wait no more
  int* err;              // global error word (nonzero: a wait gave up)
  unsigned limit;        // polls of a completion wait before it gives up
};

// polls of the drain that follows a wait that gave up (about a second)
constexpr unsigned kTcDrainPolls = 1u << 22;

// shared-memory bytes the engine needs beyond the caller's exchange buffer
template <TcForm F>
__host__ __device__ constexpr size_t tc_extra_smem(int) {
  return size_t(TcTraits<F>::parts) * 32 * TcTraits<F>::row_bytes + 16;
}
// tensor-memory columns of a CTA (a power of two >= 32)
template <int THREADS>
__host__ __device__ constexpr uint32_t tc_tmem_cols() {
  return THREADS / 128 * kTcBlockCols <= 128 ? 128 : THREADS / 128 * kTcBlockCols <= 256 ? 256 : 512;
}

// byte offset of (row, byte b within the row) in the canonical layout
template <TcForm F>
__device__ __forceinline__ uint32_t tc_off(int row, int b) {
  constexpr int RB = TcTraits<F>::row_bytes;
  constexpr int SBO = RB / 16 * 128;
  return uint32_t((row >> 3) * SBO + (b >> 4) * 128 + (row & 7) * 16 + (b & 15));
}

// bf16 bits of x rounded to nearest even, and the float they stand for
__device__ __forceinline__ uint32_t bf16_bits(float x, float& back) {
  const __nv_bfloat16 h = __float2bfloat16_rn(x);
  back = __bfloat162float(h);
  return static_cast<uint32_t>(*reinterpret_cast<const unsigned short*>(&h));
}

// set up: W^T parts, mbarrier, tensor memory; threads a multiple of 128
template <TcForm F, int THREADS>
__device__ __forceinline__ void tc_begin(TcCtx& c, unsigned char* extra, int* err, unsigned limit) {
  static_assert(THREADS % 128 == 0, "tensor-core stages use M = 128 row blocks");
  typedef TcTraits<F> TR;
  constexpr int RB = TR::row_bytes;
  c.b = extra;
  c.mbar = reinterpret_cast<uint64_t*>(c.b + TR::parts * 32 * RB);
  c.tmem_slot = reinterpret_cast<uint32_t*>(c.mbar + 1);
  c.phase = 0;
  c.dead = false;
  c.err = err;
  c.limit = limit;
  // B[n][k] = Wreal[n][k]: rows 0-15 give Yr, 16-31 Yi; columns 0-15 take
  // Xr, 16-31 Xi; W = exp(-2 pi i n k / 16); parts split from the double value
  for (int e = threadIdx.x; e < 32 * 32; e += THREADS) {
    const int n = e >> 5, k = e & 31;
    const int m = ((n & 15) * (k & 15)) & 15;
    const double cs = kTcCos16[m], sn = kTcCos16[(m + 12) & 15];
    double w;
    if (n < 16) w = k < 16 ? cs : sn;       // Wr | -Wi  (Wi = -sin)
    else w = k < 16 ? -sn : cs;             // Wi | Wr
    double rest = w;
#pragma unroll
    for (int q = 0; q < TR::parts; ++q) {
      if constexpr (F == TcForm::TF32x3) {
        const float part = tf32_round(static_cast<float>(rest));
        *reinterpret_cast<float*>(c.b + q * 32 * RB + tc_off<F>(n, k * 4)) = part;
        rest -= static_cast<double>(part);
      } else {
        const __nv_bfloat16 part = __float2bfloat16_rn(static_cast<float>(rest));
        *reinterpret_cast<__nv_bfloat16*>(c.b + q * 32 * RB + tc_off<F>(n, k * 2)) = part;
        rest -= static_cast<double>(__bfloat162float(part));
      }
    }
  }
  constexpr uint32_t cols = tc_tmem_cols<THREADS>();
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(c.tmem_slot)),
                 "n"(cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(c.mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  c.tmem = *c.tmem_slot;
}

template <int THREADS>
__device__ __forceinline__ void tc_end(TcCtx& c) {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (threadIdx.x < 32) {
    constexpr uint32_t cols = tc_tmem_cols<THREADS>();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(c.tmem), "n"(cols) : "memory");
  }
}

// One radix-16 DFT per thread, in place on v[0..15], on the tensor cores.
// Every thread of the CTA calls it together; it touches no shared memory
// but the engine's own (B, mbarrier).
template <TcForm F, int THREADS>
__device__ __forceinline__ void tc_dft16(TcCtx& c, float2 (&v)[16]) {
  typedef TcTraits<F> TR;
  constexpr int RB = TR::row_bytes;
  constexpr int KSTEPS = 32 / TR::kstep;
  constexpr uint32_t SBO = RB / 16 * 128;
  const int warp = threadIdx.x >> 5;
  // this warp's lanes (32 (warp % 4) ...) and its 128-row block's columns
  const uint32_t tbase = c.tmem + (uint32_t((warp & 3) * 32) << 16) + uint32_t((warp >> 2) * kTcBlockCols);
  // this thread's A row, K = 32 reals (Re of the 16 inputs, then Im), in parts
  if constexpr (F == TcForm::BF16x6) {
    uint32_t p0[16], p1[16], p2[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      uint32_t h[2], m[2], l[2];
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int k = 2 * j + e;
        const float x = k < 16 ? v[k].x : v[k - 16].y;
        float bh, bm, bl;
        h[e] = bf16_bits(x, bh);
        const float r1 = x - bh;               // exact
        m[e] = bf16_bits(r1, bm);
        l[e] = bf16_bits(r1 - bm, bl);         // r1 - bm exact; its bf16 rounding loses bits below 2^-24 |x|
      }
      p0[j] = h[0] | (h[1] << 16);
      p1[j] = m[0] | (m[1] << 16);
      p2[j] = l[0] | (l[1] << 16);
    }
    tmem_st16(tbase + 0, p0);
    tmem_st16(tbase + 32, p1);
    tmem_st16(tbase + 64, p2);
  } else {
    uint32_t q0[32], q1[32];
#pragma unroll
    for (int k = 0; k < 32; ++k) {
      const float x = k < 16 ? v[k].x : v[k - 16].y;
      const float hi = tf32_round(x);
      q0[k] = __float_as_uint(hi);
      q1[k] = __float_as_uint(tf32_round(x - hi));
    }
    tmem_st32(tbase + 0, q0);
    tmem_st32(tbase + 32, q1);
  }
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (threadIdx.x == 0 && !c.dead) {
    constexpr uint32_t idesc = instr_desc<F>(128, 32);
    const uint32_t bbase = smem_u32(c.b);
#pragma unroll
    for (int blk = 0; blk < THREADS / 128; ++blk) {
      const uint32_t col = c.tmem + uint32_t(blk * kTcBlockCols);
#pragma unroll
      for (int pr = 0; pr < TR::nprod; ++pr) {
#pragma unroll
        for (int ks = 0; ks < KSTEPS; ++ks) {
          // one K step of A = kstep elements = 8 columns (tf32: 1, bf16: 2 per column);
          // of B = two core matrices along K
          const uint32_t a = col + uint32_t(32 * TR::pa(pr) + 8 * ks);
          const uint64_t b = smem_desc(bbase + uint32_t(TR::pb(pr) * 32 * RB + ks * 256), 128, SBO);
          mma_tmem_a<F>(col + kTcDCol, a, b, idesc, (pr > 0 || ks > 0) ? 1u : 0u);
        }
      }
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(c.mbar))
                 : "memory");
  }
  if (!c.dead) {
    // lane 0 of each warp polls; the warp takes its verdict
    int ok = 1;
    if ((threadIdx.x & 31) == 0) {
      bool done = false;
      for (unsigned i = 0; i < c.limit && !done; ++i) done = mbar_try(smem_u32(c.mbar), c.phase);
      if (!done) {
        atomicExch(c.err, 1);
        for (unsigned i = 0; i < kTcDrainPolls && !done; ++i) done = mbar_try(smem_u32(c.mbar), c.phase);
        ok = 0;
      }
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    if (!ok) c.dead = true;
  }
  c.phase ^= 1u;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
        "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
        "=r"(r[30]), "=r"(r[31])
      : "r"(tbase + uint32_t(kTcDCol))
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = make_float2(__uint_as_float(r[k]), __uint_as_float(r[16 + k]));
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

// LineFFT over plan_with_e(L, 16) whose radix-16 stages run on the tensor
// cores; other stages (the last radix 2, 4 or 8) stay on the CUDA cores.
template <int L, TcForm F, int THREADS>
struct LineFFTTC {
  typedef LineFFT<float, L, 16> Base;
  typedef float2 V;
  static constexpr LinePlan pl = Base::pl;
  static constexpr int E = 16, P = Base::P, NS = Base::NS;
  static_assert(Base::E == 16 && pl.radix[0] == 16, "tensor-core lines start with radix 16");

  template <class Load, class XW, class XR, class AfterLoad>
  __device__ __forceinline__ static void compute(TcCtx& c, int t, const V* __restrict__ tw, Load&& load, XW&& xw,
                                                 XR&& xr, AfterLoad&& after_load, V (&v)[E]) {
#pragma unroll
    for (int r = 0; r < E; ++r) v[r] = load(t + r * P);
    after_load();
    // stage 0 reads nothing from the exchange buffer after this barrier
    __syncthreads();
    tc_dft16<F, THREADS>(c, v);
    static_for<1, NS>([&](auto s_) {
      constexpr int s = decltype(s_)::value;
      constexpr int Rp = pl.radix[s - 1];
      constexpr int R = pl.radix[s];
      constexpr int Nsp = plan_ns_before(pl, s - 1);
      constexpr int Ns = plan_ns_before(pl, s);
      constexpr int two = plan_tw_offset(pl, s);
      __syncthreads();   // every thread has read the previous exchange
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
#pragma unroll
      for (int b = 0; b < E / R; ++b) {
        const int j = t + b * P;
        const int k = j % Ns;
#pragma unroll
        for (int r = 1; r < R; ++r) v[b * R + r] = c_mul(v[b * R + r], __ldg(tw + two + (r - 1) * Ns + k));
      }
      if constexpr (R == 16) {
        tc_dft16<F, THREADS>(c, v);   // its barrier also ends this stage's exchange reads
      } else {
#pragma unroll
        for (int b = 0; b < E / R; ++b) Dft<R, 1>::run(v + b * R);
      }
    });
  }

  template <class Store>
  __device__ __forceinline__ static void emit(int t, V (&v)[E], Store&& store) {
    Base::emit(t, v, store);
  }
};

}  // namespace afg
