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
//   TcForm::TF32x3  x = hi + lo with hi = tf32(x), lo = x - hi;
//                   D = A_hi B_hi + A_hi B_lo + A_lo B_hi   (kind::tf32, K = 8 per MMA)
//   TcForm::BF16x3  the same split with bf16 parts           (kind::f16 bf16, K = 16 per MMA)
//
// Shared-memory operands use the canonical K-major layout without swizzle:
// 8-row x 16-byte core matrices, adjacent along K at LBO = 128 B, adjacent
// 8-row groups at SBO = (row bytes / 16) * 128 B.
//
// Every wait on the MMA-completion mbarrier is bounded (TcCtx::limit polls).
// A wait that gives up sets the error word, then drains: it waits again, up
// to kTcDrainPolls, for the products already issued, so no MMA still writes
// tensor memory when the kernel frees it.  After that the engine issues and
// waits no more, and the kernel always reaches its end.
#pragma once
#include <cstdint>
#include "fft_core.cuh"

namespace afg {

enum class TcForm : int { TF32x3 = 1, BF16x3 = 2 };

template <TcForm F> struct TcTraits;
template <> struct TcTraits<TcForm::TF32x3> {
  static constexpr int row_bytes = 128;     // 32 tf32 per row
  static constexpr int kstep = 8;           // K per MMA
  static constexpr uint32_t fmt = 2;        // TF32 in the A/B format fields
};
template <> struct TcTraits<TcForm::BF16x3> {
  static constexpr int row_bytes = 64;      // 32 bf16 per row
  static constexpr int kstep = 16;
  static constexpr uint32_t fmt = 1;        // BF16
};

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

template <TcForm F>
__device__ __forceinline__ void mma_issue(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  if constexpr (F == TcForm::TF32x3) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
  } else {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
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

// cos(2 pi m / 16), m = 0..15, evaluated by the compiler (sin(2 pi m / 16) =
// cos(2 pi (m - 4) / 16)); the device reads them, it never evaluates them
__constant__ double kTcCos16[16] = {
    ce_trig2pi(0, 16, false),  ce_trig2pi(1, 16, false),  ce_trig2pi(2, 16, false),  ce_trig2pi(3, 16, false),
    ce_trig2pi(4, 16, false),  ce_trig2pi(5, 16, false),  ce_trig2pi(6, 16, false),  ce_trig2pi(7, 16, false),
    ce_trig2pi(8, 16, false),  ce_trig2pi(9, 16, false),  ce_trig2pi(10, 16, false), ce_trig2pi(11, 16, false),
    ce_trig2pi(12, 16, false), ce_trig2pi(13, 16, false), ce_trig2pi(14, 16, false), ce_trig2pi(15, 16, false)};

// ----------------------------------------------------------- per-CTA context
// Shared-memory state of the engine; tc_begin() sets it up, tc_end() frees
// the tensor memory.  All threads of the CTA take part in every call.
struct TcCtx {
  unsigned char* a_hi;   // threads x row_bytes (the line exchange buffer, free during a stage)
  unsigned char* a_lo;   // threads x row_bytes
  unsigned char* b_hi;   // 32 x row_bytes: W^T high parts
  unsigned char* b_lo;   // 32 x row_bytes: W^T low parts
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

// shared-memory bytes the engine adds after the exchange buffer (which must
// hold at least threads * row_bytes)
template <TcForm F>
__host__ __device__ constexpr size_t tc_extra_smem(int threads) {
  return size_t(threads) * TcTraits<F>::row_bytes + 2 * 32 * TcTraits<F>::row_bytes + 16;
}

// byte offset of (row, byte b within the row) in the canonical layout
template <TcForm F>
__device__ __forceinline__ uint32_t tc_off(int row, int b) {
  constexpr int RB = TcTraits<F>::row_bytes;
  constexpr int SBO = RB / 16 * 128;
  return uint32_t((row >> 3) * SBO + (b >> 4) * 128 + (row & 7) * 16 + (b & 15));
}

template <TcForm F>
__device__ __forceinline__ void tc_store4(unsigned char* base, int row, int k0, float a, float b, float c, float d) {
  if constexpr (F == TcForm::TF32x3) {
    *reinterpret_cast<float4*>(base + tc_off<F>(row, k0 * 4)) = make_float4(a, b, c, d);
  } else {
    __nv_bfloat162 lo2 = __floats2bfloat162_rn(a, b), hi2 = __floats2bfloat162_rn(c, d);
    uint2 u;
    u.x = *reinterpret_cast<uint32_t*>(&lo2);
    u.y = *reinterpret_cast<uint32_t*>(&hi2);
    *reinterpret_cast<uint2*>(base + tc_off<F>(row, k0 * 2)) = u;
  }
}

// split x into the form's high and low parts, both rounded to the form's
// type (the MMA would otherwise truncate the low part's tf32 mantissa)
template <TcForm F>
__device__ __forceinline__ void tc_split(float x, float& hi, float& lo) {
  if constexpr (F == TcForm::TF32x3) {
    hi = tf32_round(x);
    lo = tf32_round(x - hi);
  } else {
    hi = __bfloat162float(__float2bfloat16_rn(x));
    lo = x - hi;
  }
}

// set up: W^T operands, mbarrier, tensor memory (cols >= 32 * blocks, a power
// of two); threads must be a multiple of 128
template <TcForm F, int THREADS>
__device__ __forceinline__ void tc_begin(TcCtx& c, unsigned char* exchange, unsigned char* extra, int* err,
                                         unsigned limit) {
  static_assert(THREADS % 128 == 0, "tensor-core stages use M = 128 row blocks");
  constexpr int RB = TcTraits<F>::row_bytes;
  c.a_hi = exchange;
  c.a_lo = extra;
  c.b_hi = extra + size_t(THREADS) * RB;
  c.b_lo = c.b_hi + 32 * RB;
  c.mbar = reinterpret_cast<uint64_t*>(c.b_lo + 32 * RB);
  c.tmem_slot = reinterpret_cast<uint32_t*>(c.mbar + 1);
  c.phase = 0;
  c.dead = false;
  c.err = err;
  c.limit = limit;
  // B[n][k] = Wreal[n][k]: rows 0-15 give Yr, 16-31 Yi; columns 0-15 take
  // Xr, 16-31 Xi; W = exp(-2 pi i n k / 16)
  for (int e = threadIdx.x; e < 32 * 32; e += THREADS) {
    const int n = e >> 5, k = e & 31;
    const int m = ((n & 15) * (k & 15)) & 15;
    const double cs = kTcCos16[m], sn = kTcCos16[(m + 12) & 15];
    double w;
    if (n < 16) w = k < 16 ? cs : sn;       // Wr | -Wi  (Wi = -sin)
    else w = k < 16 ? -sn : cs;             // Wi | Wr
    const float wf = static_cast<float>(w);
    float hi, lo;
    tc_split<F>(wf, hi, lo);
    lo = static_cast<float>(w - static_cast<double>(hi));
    if constexpr (F == TcForm::TF32x3) lo = tf32_round(lo);
    if constexpr (F == TcForm::TF32x3) {
      *reinterpret_cast<float*>(c.b_hi + tc_off<F>(n, k * 4)) = hi;
      *reinterpret_cast<float*>(c.b_lo + tc_off<F>(n, k * 4)) = lo;
    } else {
      *reinterpret_cast<__nv_bfloat16*>(c.b_hi + tc_off<F>(n, k * 2)) = __float2bfloat16_rn(hi);
      *reinterpret_cast<__nv_bfloat16*>(c.b_lo + tc_off<F>(n, k * 2)) = __float2bfloat16_rn(lo);
    }
  }
  constexpr uint32_t cols = THREADS / 128 * 32 <= 32 ? 32 : THREADS / 128 * 32 <= 64 ? 64
                           : THREADS / 128 * 32 <= 128 ? 128 : 256;
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
    constexpr uint32_t cols = THREADS / 128 * 32 <= 32 ? 32 : THREADS / 128 * 32 <= 64 ? 64
                             : THREADS / 128 * 32 <= 128 ? 128 : 256;
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(c.tmem), "n"(cols) : "memory");
  }
}

// One radix-16 DFT per thread, in place on v[0..15], on the tensor cores.
// The caller guarantees that every thread of the CTA calls it together and
// that nobody reads the exchange buffer (it holds A_hi during the call).
template <TcForm F, int THREADS>
__device__ __forceinline__ void tc_dft16(TcCtx& c, float2 (&v)[16]) {
  typedef TcTraits<F> TR;
  constexpr int RB = TR::row_bytes;
  constexpr int KSTEPS = 32 / TR::kstep;
  constexpr int BLOCK_BYTES = 128 * RB;
  const int row = threadIdx.x;
  // this thread's A row: 32 reals (Re of the 16 inputs, then Im), split
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    float x[4], h[4], l[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int k = 4 * q + j;
      x[j] = k < 16 ? v[k].x : v[k - 16].y;
      tc_split<F>(x[j], h[j], l[j]);
    }
    tc_store4<F>(c.a_hi, row, 4 * q, h[0], h[1], h[2], h[3]);
    tc_store4<F>(c.a_lo, row, 4 * q, l[0], l[1], l[2], l[3]);
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (threadIdx.x == 0 && !c.dead) {
    constexpr uint32_t idesc = instr_desc<F>(128, 32);
    constexpr uint32_t SBO = RB / 16 * 128;
    const uint32_t ah = smem_u32(c.a_hi), al = smem_u32(c.a_lo);
    const uint32_t bh = smem_u32(c.b_hi), bl = smem_u32(c.b_lo);
#pragma unroll
    for (int blk = 0; blk < THREADS / 128; ++blk) {
      const uint32_t d = c.tmem + uint32_t(blk * 32);
      const uint32_t ab = uint32_t(blk * BLOCK_BYTES);
#pragma unroll
      for (int ks = 0; ks < KSTEPS; ++ks) {
        const uint32_t ko = uint32_t(ks * 256);   // one K step = two core matrices along K
        mma_issue<F>(d, smem_desc(ah + ab + ko, 128, SBO), smem_desc(bh + ko, 128, SBO), idesc, ks > 0);
        mma_issue<F>(d, smem_desc(ah + ab + ko, 128, SBO), smem_desc(bl + ko, 128, SBO), idesc, 1);
        mma_issue<F>(d, smem_desc(al + ab + ko, 128, SBO), smem_desc(bh + ko, 128, SBO), idesc, 1);
      }
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(c.mbar))
                 : "memory");
  }
  if (!c.dead) {
    bool ok = false;
    for (unsigned i = 0; i < c.limit && !ok; ++i) ok = mbar_try(smem_u32(c.mbar), c.phase);
    if (!ok) {
      c.dead = true;
      atomicExch(c.err, 1);
      for (unsigned i = 0; i < kTcDrainPolls && !ok; ++i) ok = mbar_try(smem_u32(c.mbar), c.phase);
    }
  }
  c.phase ^= 1u;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  // this warp's 32 rows of its 128-row block: lanes 32*(warp % 4) ...
  const int warp = threadIdx.x >> 5;
  const uint32_t taddr = c.tmem + (uint32_t((warp & 3) * 32) << 16) + uint32_t((warp >> 2) * 32);
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
        "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
        "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
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
      __syncthreads();   // the previous stage's MMAs read A_hi in the exchange buffer
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
        __syncthreads();   // every thread has read this stage's inputs: A_hi may overwrite them
        tc_dft16<F, THREADS>(c, v);
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
