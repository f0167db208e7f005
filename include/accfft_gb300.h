/*
 * accfft_gb300.h - C ABI of the GB300-native AccFFT single-GPU path.
 *
 * Every entry point takes plain pointers and sizes (no C++ or framework types)
 * so it can be bound from C, ctypes, cgo or JNI.  The C++ API that mirrors
 * AccFFT's own headers (accfft_gpu.h, accfft_gpuf.h, accfft_operators_gpu.h)
 * is a thin layer over these functions.
 *
 * Conventions shared by all entry points
 *   - Grids are row-major [N0][N1][N2] (x slowest, z fastest); one process,
 *     one GPU, an MPI communicator of size one.
 *   - r2c spectra are [N0][N1][N2/2+1] complex (interleaved re, im), c2c data
 *     is [N0][N1][N2] complex.  An r2c plan is in place when data == data_out
 *     (non-NULL) at plan time; its real arrays then use rows padded to
 *     2*(N2/2+1).  Two NULL plan-time pointers make an out-of-place plan.
 *   - Transforms are unnormalised: c2r(r2c(u)) = N0*N1*N2 * u.
 *   - xyz is AccFFT's std::bitset<3> as an integer: bit 0 = x, bit 1 = y,
 *     bit 2 = z; 7 selects all axes.
 *   - timer (may be NULL) points to AccFFT's 5-slot timer; slot 4 accumulates
 *     the device time of the transform in seconds, the others are untouched.
 *   - Functions returning int return ACCFFT_C_OK (0) or an ACCFFT_C_E* code;
 *     accfft_c_last_error() describes the last failure of the calling thread.
 *   - By default every call blocks until the GPU work is done (AccFFT's
 *     contract).  accfft_c_set_stream() makes a plan enqueue asynchronously.
 *   - Arrays may be device memory or pinned host memory (cudaHostAlloc /
 *     cudaHostRegister); other host memory is rejected with ACCFFT_C_EINVAL.
 *     When an r2c input or a c2r output is pinned host memory, the plan
 *     moves it with the copy engines in 4 slab batches through a ring of
 *     three device staging slots, overlapped with the z and y kernels of the
 *     batches already staged; other arrays in host memory are reached by the
 *     kernels over the host link.
 *   - Plans are not thread-safe (one plan, one host thread at a time).
 */
#ifndef ACCFFT_GB300_H
#define ACCFFT_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define ACCFFT_C_OK 0
#define ACCFFT_C_EINVAL 1        /* invalid argument (NULL plan/pointer, bad size, wrong precision) */
#define ACCFFT_C_EUNSUPPORTED 2  /* an axis length without compiled kernels */
#define ACCFFT_C_ECUDA 3         /* CUDA runtime error (allocation, launch, execution) */
#define ACCFFT_C_ENOTBAKED 4     /* plan was not made for this transform kind */
#define ACCFFT_C_EOVERFLOW 5     /* a size does not fit the reference's int interface */

/* Plan flags beside the reference's ACCFFT_ESTIMATE/MEASURE/PATIENT (1, 2,
 * 4; accepted and ignored).  Extensions with no counterpart in the
 * reference: float r2c plans whose radix-16 line stages run on the tensor
 * cores as 32x32 real matrix products with FP32 accumulation, the data held
 * in tensor memory: ACCFFT_C_TC_TF32 splits every operand in a high and a
 * low TF32 part (3 products); ACCFFT_C_TC_BF16 in three BF16 parts (exact
 * for float data; 6 products, FP32-class accuracy).  Such plans run full
 * r2c / c2r transforms (xyz = 7) of device arrays only; x and y lengths 128,
 * 256, 512 or 1024, N2/2 128, 256 or 512. */
#define ACCFFT_C_TC_TF32 0x100u
#define ACCFFT_C_TC_BF16 0x200u
/* Double plans whose kernels compute in double-float: every value a pair
 * of floats (hi + lo, 48-bit significand) on the FP32 pipes, which on GB300
 * issue about 70x the operations per cycle of the FP64 pipe.  Arrays stay
 * IEEE double.  rel-L2 against an exact transform is about 1e-14 instead of
 * 1e-16; every transform first scans its input for the largest exponent and
 * scales its passes by that power of two, so any finite input keeps
 * normwise accuracy (entries below 2^-126 of the largest flush to zero).
 * Such plans run the r2c, c2r and c2c transforms (any xyz) and the 3-D
 * spectral operators (laplace, biharmonic, inv_laplace, inv_biharmonic,
 * heat, helmholtz, poisson with method 1: r2c, the symbol in double, c2r);
 * the single-axis transforms, grad, divergence and the finite-difference
 * Poisson method stay with plain double plans.  The exponent lives in one
 * word of the plan, so two transforms of one plan must not overlap on the
 * GPU. */
#define ACCFFT_C_F64_DF 0x400u

typedef struct accfft_c_plan accfft_c_plan; /* opaque */

/* --- library --------------------------------------------------------- */
const char* accfft_c_last_error(void);
/* the ACCFFT_C_E* code of that failure (ACCFFT_C_OK after a successful
 * call): plan creation reports failure by returning NULL, this says why */
int accfft_c_last_error_code(void);
int accfft_c_version(void);
/* 1 if an axis of this length has compiled kernels (complex length for
 * c2c axes; for the real z axis of an r2c plan the check is on N2/2) */
int accfft_c_length_supported(int len);
/* 1 if a line of this length runs on the generic kernels (lengths up to
 * 4096 whose prime factors are at most 31; the real z axis of an r2c plan
 * as its full length N2, odd N2 included).  Plans whose axes are all either
 * compiled or generic are accepted; an axis on the generic kernels limits
 * the plan to the transforms (any xyz, device arrays) and the 3-D spectral
 * operators, which then run as r2c, a symbol pass and c2r; such plans are
 * float or double (not double-float or tensor-core) and are not tuned. */
int accfft_c_length_generic(int len);
/* the compiled radix plan of a line length for the arithmetic `precision`
 * (0 float, 1 double, 2 double-float): first radix *E, threads per line *P
 * and the stage radices in radices[0..] (at most 16); returns the number of
 * stages (0 for length 1), -1 when the length has no plan or an argument is
 * invalid.  Needs no plan and no GPU. */
int accfft_c_line_plan(int len, int precision, int* E, int* P, int* radices);
/* kernels launched by this process through the library (for audits) */
unsigned long long accfft_c_kernel_launches(void);
/* programmatic dependent launch of the pass kernels (each pass waits in
 * hardware for the pass before it): 0 off; 1 the next pass is released as
 * this one's CTAs finish (hides the launch latency; the default); 2 it is
 * released as they start, so its CTAs wait on the SMs this pass's last wave
 * leaves idle.  ACCFFT_GB300_PDL=0|1|2 in the environment sets the start
 * value; mode >= 0 sets it for the process, -1 only queries; returns the
 * previous mode. */
int accfft_c_set_pdl(int mode);
/* extension: every device-side wait of the library's kernels is bounded (the
 * tensor-core forms wait for their matrix products; the persistent z+y
 * schedule's items wait for the items of their slab).  A wait gives up after
 * `polls` polls (the default, 2^22, is about half a second), sets the plan's
 * error word and lets the kernel finish without the missing data; the call
 * (or, for a non-blocking call, the plan's next blocking or timed call, or
 * accfft_c_check) then returns ACCFFT_C_ECUDA and its results are not valid.
 * The reference's execute has no failure path of this kind (its waits are
 * cuFFT's and the runtime's).  polls < 0 restores the default; the setting
 * is per process; returns the previous value. */
long long accfft_c_set_wait_limit(long long polls);
/* extension: wait for everything enqueued by the plan and report a device-side
 * wait that gave up since the plan's last blocking, timed or checked call
 * (ACCFFT_C_ECUDA); ACCFFT_C_OK otherwise */
int accfft_c_check(accfft_c_plan* plan);

/* --- local sizes ------------------------------------------------------
 * Replaces dfft_get_local_size_t (src/accfft_common.cpp:49-91),
 * accfft_local_size_dft_r2c_t (src/accfft_common.cpp:98-192) and
 * accfft_local_size_dft_c2c_t (src/accfft_common.cpp:203-256) at P = 1.
 * real_bytes is sizeof(double) or sizeof(float).  The return value is the
 * byte count the reference would return (alloc_max), as 64-bit. */
long long accfft_c_dfft_get_local_size(int N0, int N1, int tuple, int isize[3], int istart[3],
                                       int real_bytes);
long long accfft_c_local_size_dft_r2c(const int n[3], int isize[3], int istart[3], int osize[3],
                                      int ostart[3], int real_bytes);
long long accfft_c_local_size_dft_c2c(const int n[3], int isize[3], int istart[3], int osize[3],
                                      int ostart[3], int real_bytes);

/* --- plans ------------------------------------------------------------
 * Replace accfft_plan_dft_3d_r2c_gpu (src/accfft_gpu.cpp:77-442),
 * accfft_plan_dft_3d_c2c_gpu (src/accfft_gpu.cpp:704-931) and their float
 * twins (src/accfft_gpuf.cpp:74, :697).  Return NULL on failure. */
accfft_c_plan* accfft_c_plan_dft_3d_r2c_gpu(const int n[3], double* data, double* data_out, unsigned flags);
accfft_c_plan* accfft_c_plan_dft_3d_r2c_gpuf(const int n[3], float* data, float* data_out, unsigned flags);
accfft_c_plan* accfft_c_plan_dft_3d_c2c_gpu(const int n[3], double* data, double* data_out, unsigned flags);
accfft_c_plan* accfft_c_plan_dft_3d_c2c_gpuf(const int n[3], float* data, float* data_out, unsigned flags);
/* Replaces accfft_destroy_plan_gpu (src/accfft_gpu.cpp:1142-1192); frees the plan itself too. */
void accfft_c_destroy_plan(accfft_c_plan* plan);
/* kind: 1 = r2c, 2 = c2c; is_double: 1 for the double plans */
int accfft_c_plan_info(const accfft_c_plan* plan, int n[3], int* kind, int* is_double, int* inplace,
                       long long* alloc_max);
/* extension: how an r2c plan runs its z and y passes: 0 = one kernel per
 * pass over the whole grid (default), 1 = one thread-block-cluster kernel per
 * x-slab doing both, 2 = one persistent kernel whose CTAs take z rows and y
 * columns slab by slab with per-slab dependency counters, so the second pass
 * of a slab reads it from L2 (ACCFFT_C_EUNSUPPORTED when the grid has no
 * such kernel) */
int accfft_c_set_zy_schedule(accfft_c_plan* plan, int mode);
/* extension: pass order of full r2c / c2r transforms (xyz = 111) of device
 * arrays.  0 = the reference's order (src/accfft_gpu.cpp:470-603): z r2c,
 * then y and x passes on the [N0][N1][N2/2+1] spectrum, whose rows of N2/2+1
 * complex are not 16-byte aligned.  1 = packed: the y and x passes run on the
 * real field viewed as complex [N0][N1][N2/2] (aligned rows) in the plan
 * scratch, and one z pass over mirror-paired lines (x, y) / (-x, -y)
 * completes the real transform and writes the natural spectrum row by row;
 * c2r runs the same passes backwards and only reads its input.  Same
 * results to rounding.  Out-of-place float and double plans only
 * (ACCFFT_C_EUNSUPPORTED otherwise), where it is the default;
 * ACCFFT_GB300_ORDER=natural in the environment makes 0 the default. */
int accfft_c_set_pass_order(accfft_c_plan* plan, int order);
/* ACCFFT_MEASURE (the reference's default flag: tune at plan creation,
 * src/accfft_gpu.cpp:341-382) on a float r2c plan times the radix / tile
 * variants of its y, x, z r2c and z c2r passes on the plan's scratch and a
 * temporary spectrum (variant 0 = default; 1 = half the columns or the other
 * line count per CTA; 2 = the next smaller first radix; 3 = for y and x,
 * the default tile with 16-byte loads and stores; 4 = for y and x of 512
 * and 1024, one persistent CTA a SM with three column tiles in flight
 * through tensor copies, its waits bounded and reported like the
 * tensor-core ones, see accfft_c_check) and keeps the
 * fastest; the choice is cached per process by grid and pass order, so plans
 * of one grid run the same kernels.  ACCFFT_ESTIMATE keeps the defaults.
 * accfft_c_plan_tuning reports, for y, x, z r2c and z c2r, the variant, its
 * first radix and its tile width (columns or lines per CTA; 0 where the
 * length has no variants); returns 1 when the plan was tuned, else 0.
 * accfft_c_set_variants sets the four variants by hand (float r2c plans;
 * ACCFFT_C_EUNSUPPORTED for a variant the length does not have).  Batches
 * (below) run the default variants. */
int accfft_c_plan_tuning(const accfft_c_plan* plan, int variant[4], int radix[4], int tile[4]);
int accfft_c_set_variants(accfft_c_plan* plan, const int variant[4]);
/* extension: per-kernel device times.  With profiling on, every kernel the
 * plan launches is bracketed by CUDA events on its stream;
 * accfft_c_profile_read waits for them and returns, per pass label ("z_r2c",
 * "y", "x", "x_inv", "y_inv", "z_c2r", "x_sym", "x_deriv", "h2d", ...;
 * host copies are included), the launch count and
 * total milliseconds since the previous read (labels: 32 bytes each).  The
 * return value is the number of labels written. */
int accfft_c_set_profiling(accfft_c_plan* plan, int on);
int accfft_c_profile_read(accfft_c_plan* plan, int max_entries, char* labels, long long* counts, double* total_ms);
/* extension: enqueue on `stream` (a cudaStream_t); blocking = 0 returns
 * without waiting (timer slots are then not updated).  A plan's calls share
 * its scratch spectrum (and a double-float plan's exponent word): calls of
 * one plan must not overlap on the GPU, so run concurrent transforms with
 * one plan each. */
int accfft_c_set_stream(accfft_c_plan* plan, void* stream, int blocking);

/* --- transforms -------------------------------------------------------
 * Replace accfft_execute_r2c_gpu (src/accfft_gpu.cpp:635-649),
 * accfft_execute_c2r_gpu (:661-675), accfft_execute_gpu (:444-623),
 * accfft_execute_c2c_gpu (:943-1136) and the float twins
 * (src/accfft_gpuf.cpp:443, :632, :656, :935).  NULL data pointers select
 * the pointers given at plan time.  Unlike the reference, an out-of-place
 * c2r or backward c2c leaves its input unchanged. */
int accfft_c_execute_r2c_gpu(accfft_c_plan* plan, double* data, double* data_out, double* timer, unsigned xyz);
int accfft_c_execute_c2r_gpu(accfft_c_plan* plan, double* data, double* data_out, double* timer, unsigned xyz);
int accfft_c_execute_gpu(accfft_c_plan* plan, int direction, double* data, double* data_out, double* timer,
                         unsigned xyz);
int accfft_c_execute_c2c_gpu(accfft_c_plan* plan, int direction, double* data, double* data_out, double* timer,
                             unsigned xyz);
int accfft_c_execute_r2c_gpuf(accfft_c_plan* plan, float* data, float* data_out, double* timer, unsigned xyz);
int accfft_c_execute_c2r_gpuf(accfft_c_plan* plan, float* data, float* data_out, double* timer, unsigned xyz);
int accfft_c_execute_gpuf(accfft_c_plan* plan, int direction, float* data, float* data_out, double* timer,
                          unsigned xyz);
int accfft_c_execute_c2c_gpuf(accfft_c_plan* plan, int direction, float* data, float* data_out, double* timer,
                              unsigned xyz);

/* Single-axis real transforms, replacing accfft_execute_{r2c,c2r}_{z,y,x}_gpu_t
 * (src/accfft_gpu.cpp:1212-1604; float src/accfft_gpuf.cpp:1197-1572).
 * Spectrum layouts: z -> [N0][N1][N2/2+1], y -> [N0][N1/2+1][N2],
 * x -> [N0/2+1][N1][N2].  axis: 0 = x, 1 = y, 2 = z.  Double plans take
 * double arrays, float plans float arrays (passed as void*).  The x and y
 * transforms use unpadded [N0][N1][N2] real arrays (as the reference's), the
 * z transform the plan's real layout; c2r leaves its input unchanged. */
int accfft_c_execute_r2c_axis(accfft_c_plan* plan, int axis, const void* data, void* data_out, double* timer);
int accfft_c_execute_c2r_axis(accfft_c_plan* plan, int axis, const void* data, void* data_out, double* timer);

/* --- spectral operators (r2c plans) -----------------------------------
 * Replace accfft_{grad,laplace,divergence,biharmonic}_gpu[f]
 * (src/operators_gpu.cpp:85-135, src/operators_gpu.txx:72-609,
 * src/operators_gpuf.cpp:93-143).  inv_laplace and inv_biharmonic have no
 * GPU version in the reference; they follow the CPU kernels
 * mult_wave_number_inv_laplace (src/operators.txx:276-333) and
 * mult_wave_number_inv_biharmonic (src/operators.txx:336-388).
 * Arrays have the plan's precision and real layout.  grad's xyz selects the
 * components (NULL outputs are allowed for unselected ones). */
int accfft_c_grad(accfft_c_plan* plan, void* A_x, void* A_y, void* A_z, const void* A, unsigned xyz, double* timer);
int accfft_c_grad_slow(accfft_c_plan* plan, void* A_x, void* A_y, void* A_z, const void* A, unsigned xyz,
                       double* timer);
int accfft_c_laplace(accfft_c_plan* plan, void* LA, const void* A, double* timer);
int accfft_c_divergence(accfft_c_plan* plan, void* divA, const void* A_x, const void* A_y, const void* A_z,
                        double* timer);
int accfft_c_divergence_slow(accfft_c_plan* plan, void* divA, const void* A_x, const void* A_y, const void* A_z,
                             double* timer);
int accfft_c_biharmonic(accfft_c_plan* plan, void* BA, const void* A, double* timer);
int accfft_c_inv_laplace(accfft_c_plan* plan, void* invLA, const void* A, double* timer);
int accfft_c_inv_biharmonic(accfft_c_plan* plan, void* invBA, const void* A, double* timer);

/* --- spectral solvers -------------------------------------------------------
 * No GPU counterpart in the reference.  With the operators' wave numbers
 * (w = i, i - N above N/2, 0 at N/2 on each axis) and |k|^2 = wx^2 + wy^2 + wz^2:
 *   heat:      out = c2r(exp(-t |k|^2) r2c(in)) / N   - the exact solution at
 *              time t of u_t = laplace(u) from u(0) = in (as steps/step6 checks)
 *   helmholtz: out = c2r(r2c(in) / (alpha + |k|^2)) / N - solves
 *              (alpha - laplace) out = in; 0 where alpha + |k|^2 = 0, so alpha = 0
 *              gives the zero-mean Poisson solution -inv_laplace (as steps/step4)
 * Each is one fused operator: z r2c, y, x forward * symbol * x backward, y, z c2r. */
int accfft_c_heat(accfft_c_plan* plan, void* out, const void* in, double t, double* timer);
int accfft_c_helmholtz(accfft_c_plan* plan, void* out, const void* in, double alpha, double* timer);
/* extension: the Poisson solve of steps/step4 (steps/step4/step4_gpu.cpp:620-650,
 * filter steps/step4/kernels.cu:24-110) as one fused operator on the unit
 * cube (grid x_i = i / N_i): phi = c2r(r2c(rho) / S) / N with the zero mode
 * set to 0.  method 0: S = 2 sum_i (cos(2 pi k_i / N_i) - 1) N_i^2, the
 * finite-difference Laplacian; method 1: S = -4 pi^2 |k|^2 with k_i folded
 * above N_i / 2 (no Nyquist filter). */
int accfft_c_poisson(accfft_c_plan* plan, void* phi, const void* rho, int method, double* timer);

/* --- adjoints ------------------------------------------------------------
 * No counterpart in the reference; they are the backward passes of the
 * autograd layer (accfft_gb300/autograd.py).  With R the unnormalised 3-D r2c
 * of the plan and w the half-spectrum weights (1 on the kz = 0 and
 * kz = N2/2 planes, 2 on the interior planes, so that c2r(Y) = Re sum w Y e^{+i theta}):
 *   r2c_adjoint:  du = R^T dX = Re sum_k dX_k e^{+i theta}  = c2r(dX / w)
 *   c2r_adjoint:  dY = w * R dx                            = w * r2c(dx)
 *   grad_adjoint: out = -(d g_x/dx + d g_y/dy + d g_z/dz)  (the transpose of grad)
 *   divergence_adjoint: (a_x, a_y, a_z) = -grad(d)          (the transpose of divergence)
 * The weights are applied inside the z kernels; no extra pass runs. */
int accfft_c_r2c_adjoint(accfft_c_plan* plan, const void* dX, void* du, double* timer);
int accfft_c_c2r_adjoint(accfft_c_plan* plan, const void* dx, void* dY, double* timer);
int accfft_c_grad_adjoint(accfft_c_plan* plan, void* out, const void* g_x, const void* g_y, const void* g_z,
                          double* timer);
int accfft_c_divergence_adjoint(accfft_c_plan* plan, void* a_x, void* a_y, void* a_z, const void* d, double* timer);

/* --- batches (extension; no counterpart in the reference) ---------------
 * Many independent transforms of uneven sizes in one pass-by-pass schedule.
 * While a float r2c plan records (accfft_c_batch_record(b, plan, 1)), its
 * execute and 3-D operator calls append their passes to the batch as one
 * instance instead of launching them (r2c, c2r in either pass order,
 * laplace, biharmonic, inv_laplace, inv_biharmonic, heat, helmholtz,
 * poisson, grad_slow; other calls return ACCFFT_C_EUNSUPPORTED).
 * accfft_c_batch_finalize groups level k (the k-th pass of every instance)
 * by pass kind and line length and uploads one descriptor table per group;
 * accfft_c_batch_run launches one persistent kernel per group on eight
 * streams of the batch forked from `stream` and joined before it returns;
 * each group waits only for the groups of the level before that hold its
 * instances' previous passes (capturable into a CUDA graph).  Line
 * lengths up to 256.  One instance per plan (the plan's scratch belongs to
 * it); the arrays given to the recorded calls must stay valid and distinct
 * between instances; a batch runs one call at a time. */
typedef struct accfft_c_batch accfft_c_batch;
accfft_c_batch* accfft_c_batch_create(void);
void accfft_c_batch_destroy(accfft_c_batch* batch);
int accfft_c_batch_record(accfft_c_batch* batch, accfft_c_plan* plan, int on);
int accfft_c_batch_finalize(accfft_c_batch* batch);
int accfft_c_batch_run(accfft_c_batch* batch, void* stream);
int accfft_c_batch_info(const accfft_c_batch* batch, int* instances, int* levels, int* launches, int* tasks);

/* --- Laplacian without device allocation ------------------------------
 * No counterpart in the reference.  For callers that may not call cudaMalloc
 * (a plugin in an application whose memory manager has reserved the whole
 * device, a latency-bound loop where an allocation could stall the GPU) and
 * therefore cannot create a plan.  Computes the same result as
 * accfft_c_laplace with a float r2c plan on out-of-place [N0][N1][N2] arrays
 * (N2 even), using a library-owned array of 64 MiB per device instead of
 * allocating: grids whose half spectrum plus twiddle tables exceed 64 MiB
 * (e.g. beyond 256x256x240) are rejected with ACCFFT_C_EINVAL.  Nothing is
 * allocated on the device and nothing is freed.
 * The first call on a device performs a one-time set-up; make it before any
 * stream capture.  Every call reuses the same array, so calls that overlap on
 * the GPU race.  `stream` is a cudaStream_t of the current device (NULL: the
 * default stream; a stream of another device is refused with
 * ACCFFT_C_EINVAL); the call returns when the result is complete. */
int accfft_c_laplace_gpuf_noalloc(const int n[3], float* LA, const float* A, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* ACCFFT_GB300_H */
