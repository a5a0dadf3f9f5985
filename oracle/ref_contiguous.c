/* ref_contiguous.c — TEST AND CPU-BASELINE INFRASTRUCTURE ONLY.
 *
 * FP32 CPU restatement of the reference's own GPU algorithm for the path,
 * FFT_OpenCL_Contiguous<float>, used as the timed "reference algorithm on
 * the host cores" baseline (the reference itself ran this algorithm on a CPU
 * OpenCL device, Measurements.txt:492-535).  The OpenCL original cannot be
 * built here (cl.hpp:141-147 needs <CL/opencl.h> and <GL/gl.h>), so its
 * generated kernels are restated as plain C loops:
 *
 *   plan       FFT_OpenCL_Contiguous.h:54-61  BGs = [16]*floor(log2 L/4) (+ 2^(log2 L mod 4))
 *              OpenCLFFTAlgorithm.h:9-12      A_q = prod_{i<q} B_i, N_q = A_q * B_q
 *   pass q     FFT_OpenCL_Contiguous.h:167-180
 *              work-item j: g = j / (L/N_q), z = j mod (L/N_q) + batch*L
 *              x_s = in[z + (L/N_q)(B_q g + s)];  q > 1: x_s *= unit(-s g, N_q)
 *              y   = local B_q-point DFT;  out[z + (L/N_q)(g + A_q h)] = y_h
 *   local DFT  OpenCLFFTAlgorithm.h:14-43: log2(B_q) radix-2 Stockham stages in
 *              registers, constant twiddles KomplexUnit(-gL sL, NL) printed with
 *              6 significant digits (KernelGenerator.h:53-69), trivial ones as
 *              swaps/negations (KernelGenerator.h:107-119)
 *   unit(n,d)  KernelGenerator.h:48: (cos, sin)(6.28319f/d * n) in float
 *   execute    FFT_OpenCL_Contiguous.h:97-142: ping-pong between two buffers;
 *              backward = conj -> forward -> conj (applied here to every
 *              transform; the original conjugates only batch 0, :100-102).
 *
 * Layout: interleaved complex64 (the layout the benchmark configurations
 * use) instead of the reference's 32+32 block-planar host layout; the index
 * arithmetic of the passes is unchanged by that.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  float re, im;
} c32;

static int ceilog2(int64_t n) {
  int r = 0;
  for (int64_t v = 1; v < n; v *= 2) r++;
  return r;
}

/* KomplexUnit(num, den) as emitted into the kernel source: cos/sin of
 * 2 pi num / den in double, streamed with 6 significant digits, read back as
 * a float literal. */
static c32 literal_unit(int num, int den) {
  char buf[64];
  c32 r;
  snprintf(buf, sizeof buf, "%g", cos((2 * M_PI * num) / den));
  r.re = strtof(buf, NULL);
  snprintf(buf, sizeof buf, "%g", sin((2 * M_PI * num) / den));
  r.im = strtof(buf, NULL);
  return r;
}

/* KomplexConstMultiplication(KomplexUnit(num, den), b): +-1 and +-i become
 * swaps / negations, anything else a multiplication by the literal. */
typedef struct {
  int kind; /* 0: *1, 1: *-1, 2: *i, 3: *-i, 4: literal */
  c32 lit;
} const_tw;

static const_tw make_const(int num, int den) {
  const_tw t;
  int m = ((num % den) + den) % den;
  t.lit = (c32){1.f, 0.f};
  if ((4 * m) % den == 0) {
    if (m == 0) t.kind = 0;
    else if (2 * m == den) t.kind = 1;
    else if (4 * m == den) t.kind = 2;
    else t.kind = 3;
  } else {
    t.kind = 4;
    t.lit = literal_unit(num, den);
  }
  return t;
}

static inline c32 apply_const(const_tw t, c32 b) {
  switch (t.kind) {
    case 0: return b;
    case 1: return (c32){-b.re, -b.im};
    case 2: return (c32){-b.im, b.re};
    case 3: return (c32){b.im, -b.re};
    default: return (c32){t.lit.re * b.re - t.lit.im * b.im, t.lit.re * b.im + t.lit.im * b.re};
  }
}

/* unit(n, d) of the generated kernel: 2*M_PI streamed at default precision. */
static inline c32 runtime_unit(int n, int d) {
  const float f = 6.28319f / (float)d;
  return (c32){cosf(f * (float)n), sinf(f * (float)n)};
}

/* The constants the generator bakes into a local B-point DFT (B <= 16):
 * stage qL (1-based), group gL: KomplexUnit(-gL, 2^qL); and KomplexUnit(-1, 2). */
static const_tw g_stage_tw[5][8];
static const_tw g_minus_one;
static pthread_once_t g_once = PTHREAD_ONCE_INIT;
static void init_consts(void) {
  for (int qL = 1; qL <= 4; qL++)
    for (int gL = 0; gL < (1 << (qL - 1)); gL++) g_stage_tw[qL][gL] = make_const(-gL, 1 << qL);
  g_minus_one = make_const(-1, 2);
}

/* Local B-point DFT: radix-2 Stockham with AL = [1,2,4,..], NL = [2,4,8,..]
 * (OpenCLFFTAlgorithm.h:18-40 with BL = [2,2,..]). */
static void local_dft(c32* buf0, c32* buf1, int B) {
  c32* bufs[2] = {buf0, buf1};
  int kL = ceilog2(B);
  for (int qL = 1; qL <= kL; qL++) {
    c32* src = bufs[(qL ^ 1) & 1];
    c32* dst = bufs[qL & 1];
    int AL = 1 << (qL - 1), NL = 1 << qL, per = B / NL;
    for (int gL = 0; gL < AL; gL++)
      for (int zL = 0; zL < per; zL++) {
        c32 s0 = src[per * (2 * gL + 0) + zL];
        c32 s1 = apply_const(g_stage_tw[qL][gL], src[per * (2 * gL + 1) + zL]);
        dst[per * (gL + AL * 0) + zL] = (c32){s0.re + s1.re, s0.im + s1.im};
        c32 m1 = apply_const(g_minus_one, s1);
        dst[per * (gL + AL * 1) + zL] = (c32){s0.re + m1.re, s0.im + m1.im};
      }
  }
  if (kL & 1) memcpy(buf0, buf1, sizeof(c32) * (size_t)B);
}

typedef struct {
  const c32* in;
  c32* out;
  int64_t L, i0, i1; /* work items [i0, i1) over all transforms */
  int B, A, Nq, first;
} pass_job;

static void* pass_worker(void* arg) {
  pass_job* p = (pass_job*)arg;
  int64_t L = p->L, per = L / p->Nq, items = L / p->B;
  c32 x[16], y[16];
  for (int64_t gi = p->i0; gi < p->i1; gi++) {
    int64_t bi = gi / items, j = gi - bi * items;
    int64_t g = j / per, z = j - per * g + bi * L;
    for (int s = 0; s < p->B; s++) x[s] = p->in[z + per * (p->B * g + s)];
    if (!p->first)
      for (int s = 1; s < p->B; s++) {
        c32 w = runtime_unit((int)(-s * g), p->Nq);
        c32 v = x[s];
        x[s] = (c32){v.re * w.re - v.im * w.im, v.re * w.im + v.im * w.re};
      }
    local_dft(x, y, p->B);
    for (int h = 0; h < p->B; h++) p->out[z + per * (g + (int64_t)p->A * h)] = x[h];
  }
  return NULL;
}

/* Batched forward (sign -1) or backward (+1) transform of interleaved
 * complex64 data; `work` holds batch*L elements of scratch. */
int ref_contiguous_fft(const float* inp, float* outp, float* workp, int64_t L, int64_t batch, int sign,
                       int nthreads) {
  if (L < 1 || (L & (L - 1))) return -1;
  int64_t total = L * batch;
  c32* in = (c32*)inp;
  c32* out = (c32*)outp;
  c32* work = (c32*)workp;
  if (L == 1) {
    memmove(out, in, sizeof(c32) * (size_t)total);
    return 0;
  }
  pthread_once(&g_once, init_consts);
  int lg = ceilog2(L), nb = lg / 4, rem = lg % 4;
  int B[16], nq = 0;
  for (int i = 0; i < nb; i++) B[nq++] = 16;
  if (rem) B[nq++] = 1 << rem;
  /* the buffers ping-pong: pass q reads bufs[q & 1]; the result must land in out */
  c32* bufs[2];
  bufs[nq & 1] = out;
  bufs[(nq & 1) ^ 1] = work;
  memcpy(bufs[0], in, sizeof(c32) * (size_t)total);
  if (sign > 0)
    for (int64_t i = 0; i < total; i++) bufs[0][i].im = -bufs[0][i].im;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  int A = 1;
  for (int q = 0; q < nq; q++) {
    int Nq = A * B[q];
    pass_job jobs[256];
    pthread_t th[256];
    int64_t items = batch * (L / B[q]);
    int nt = nthreads;
    if (nt > items) nt = (int)items;
    for (int t = 0; t < nt; t++) {
      jobs[t] = (pass_job){bufs[q & 1], bufs[(q & 1) ^ 1], L, items * t / nt, items * (t + 1) / nt, B[q], A, Nq, q == 0};
    }
    if (nt == 1) {
      pass_worker(&jobs[0]);
    } else {
      for (int t = 0; t < nt; t++) pthread_create(&th[t], NULL, pass_worker, &jobs[t]);
      for (int t = 0; t < nt; t++) pthread_join(th[t], NULL);
    }
    A = Nq;
  }
  if (sign > 0)
    for (int64_t i = 0; i < total; i++) out[i].im = -out[i].im;
  return 0;
}
