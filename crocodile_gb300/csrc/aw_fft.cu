// AW kernel generation by FFT (the complex64 table of aw_kernel_fn,
// crocodile/synthesis.py:701-734, for 16 x 16 AW kernels and w sub-kernels of
// support S <= 16).
//
// out[k, f] = convolve2d(akern_k, W[w_k, f], 'same') is the middle 16 x 16
// (offset o = (S - 1) / 2) of the full 31 x 31 linear convolution, which a
// 32 x 32 circular convolution of the zero-padded inputs reproduces exactly.
// So with FA_k = FFT32(akern_k) / 1024 and FW_wf = FFT32(W[w, f]) (batched
// cuFFT, complex64), out[k, f] = crop(IFFT32(FA_k * FW_wf)).  The direct form
// costs 256 x (taps <= 256) complex MACs per output sub-kernel; this one a
// 1024-point product and a pruned 32 x 32 inverse transform.
//
// k_aw_fftconv (complex128 tables; complex64 ones run k_aw_fftconv_f below):
// one CTA per AW key, FA_k in shared memory, each warp takes sub-kernels f
// in turn.  Lane = column k2: the warp loads FW_wf row by row
// (coalesced), multiplies by FA_k, runs a 32-point decimation-in-frequency
// inverse FFT over k1 in registers (twiddle indices compile-time, table in
// constant memory), keeps the 16 rows n1 of the crop, and transforms each of
// them across the lanes with butterflies over __shfl_xor (per-lane twiddles
// fixed per stage).  Output n2 lands on lane bitrev5(n2).
#include <cufft.h>

#include <cmath>

#include "cg_internal.cuh"
#include "fft32.h"

namespace cg {

int fft_plan(int batch, int H, int W, cufftType type, cufftHandle *out);

__constant__ float2 c_tw32[32];    // exp(+2 pi i t / 32)
__constant__ double2 c_tw32d[32];  // the same in FP64 (complex128 tables)

namespace {

// the complex type of each precision
template <typename R> struct Cx;
template <> struct Cx<float> {
  typedef float2 T;
  static __device__ __forceinline__ T tw(int i) { return c_tw32[i]; }
};
template <> struct Cx<double> {
  typedef double2 T;
  static __device__ __forceinline__ T tw(int i) { return c_tw32d[i]; }
};

__host__ __device__ constexpr int bitrev5(int i) {
  return ((i & 1) << 4) | ((i & 2) << 2) | (i & 4) | ((i & 8) >> 2) | ((i & 16) >> 4);
}

template <int H, typename T>
__device__ __forceinline__ void dif_stage(T (&x)[32]) {
#pragma unroll
  for (int b = 0; b < 32; b += 2 * H) {
#pragma unroll
    for (int j = 0; j < H; ++j) {
      const T a = x[b + j], c = x[b + j + H];
      x[b + j].x = a.x + c.x;
      x[b + j].y = a.y + c.y;
      T d;
      d.x = a.x - c.x;
      d.y = a.y - c.y;
      if (j == 0) {
        x[b + j + H] = d;
      } else {
        const T w = Cx<decltype(d.x)>::tw(j * (16 / H));
        x[b + j + H].x = d.x * w.x - d.y * w.y;
        x[b + j + H].y = d.x * w.y + d.y * w.x;
      }
    }
  }
}

// 32-point inverse DFT (exp(+2 pi i), unnormalised): natural order in,
// bit-reversed order out (x[i] holds output bitrev5(i))
template <typename T>
__device__ __forceinline__ void idft32_dif(T (&x)[32]) {
  dif_stage<16>(x);
  dif_stage<8>(x);
  dif_stage<4>(x);
  dif_stage<2>(x);
  dif_stage<1>(x);
}

// FA: akern [nk][16][16] zero-padded to [nk][32][32] and scaled by 1/1024
template <typename T>
__global__ void k_pad_akern(const T *__restrict__ akern, int nk, T *__restrict__ fa) {
  const int64_t total = (int64_t)nk * 1024;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(e >> 10), r = (int)((e >> 5) & 31), c = (int)(e & 31);
    T v;
    v.x = v.y = 0;
    if (r < 16 && c < 16) {
      v = akern[((int64_t)k * 16 + r) * 16 + c];
      v.x *= (decltype(v.x))(1.0 / 1024.0);
      v.y *= (decltype(v.x))(1.0 / 1024.0);
    }
    fa[e] = v;
  }
}

// FW: W [nWQ][S][S] (FP64) zero-padded to [nWQ][32][32] (rounded to FP32 for
// complex64 tables)
template <typename T>
__global__ void k_pad_w(const double2 *__restrict__ W, int64_t nwq, int S, T *__restrict__ fw) {
  const int64_t total = nwq * 1024;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t g = e >> 10;
    const int r = (int)((e >> 5) & 31), c = (int)(e & 31);
    T v;
    v.x = v.y = 0;
    if (r < S && c < S) {
      const double2 d = W[(g * S + r) * S + c];
      v.x = (decltype(v.x))d.x;
      v.y = (decltype(v.x))d.y;
    }
    fw[e] = v;
  }
}

template <typename T, int S>
__global__ void __launch_bounds__(256, sizeof(T) == 8 ? 2 : 1) k_aw_fftconv(
    const T *__restrict__ fa, const T *__restrict__ fw, int nW, int QQ,
    const int32_t *__restrict__ wi, T *__restrict__ out, int32_t *status) {
  __shared__ T sfa[32][33];
  constexpr int o = (S - 1) / 2;
  const int k = blockIdx.x;
  const int w = wi[k];
  if (w < 0 || w >= nW) {
    if (threadIdx.x == 0) atomicAdd(&status[ST_INDEX], 1);
    return;
  }
  if ((status[ST_RANGE] | status[ST_INDEX]) != 0) return;
  for (int t = threadIdx.x; t < 1024; t += blockDim.x)
    sfa[t >> 5][t & 31] = fa[(int64_t)k * 1024 + t];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  typedef decltype(sfa[0][0].x) R;
  // this lane's twiddle in each across-lane stage (distance d = 16 .. 1)
  T tw[5];
#pragma unroll
  for (int st = 0; st < 5; ++st) {
    const int d = 16 >> st;
    tw[st] = Cx<R>::tw((lane & (d - 1)) * (16 / d));
  }
  const int n2 = bitrev5(lane);
  const bool keep = n2 >= o && n2 < o + 16;
  for (int f = warp; f < QQ; f += 8) {
    const T *src = fw + ((int64_t)w * QQ + f) * 1024;
    T x[32];
#pragma unroll
    for (int k1 = 0; k1 < 32; ++k1) {
      const T b = src[k1 * 32 + lane];
      const T a = sfa[k1][lane];
      x[k1].x = a.x * b.x - a.y * b.y;
      x[k1].y = a.x * b.y + a.y * b.x;
    }
    idft32_dif(x);  // over k1: x[i] = Y[bitrev5(i)][lane]
    T *dst = out + ((int64_t)k * QQ + f) * 256;
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      T v = x[bitrev5(o + r)];  // row n1 = o + r
#pragma unroll
      for (int st = 0; st < 5; ++st) {
        const int d = 16 >> st;
        T p;
        p.x = __shfl_xor_sync(0xffffffffu, v.x, d);
        p.y = __shfl_xor_sync(0xffffffffu, v.y, d);
        if (lane & d) {  // upper element: (partner - v) * twiddle
          T q;
          q.x = p.x - v.x;
          q.y = p.y - v.y;
          v.x = q.x * tw[st].x - q.y * tw[st].y;
          v.y = q.x * tw[st].y + q.y * tw[st].x;
        } else {
          v.x = v.x + p.x;
          v.y = v.y + p.y;
        }
      }
      if (keep) dst[r * 16 + (n2 - o)] = v;
    }
  }
}

// The complex64 form with 16-point register transforms (fft32.h) and one
// transpose through shared memory in place of the shuffled row pass: per
// sub-kernel about 800 warp instructions against 1,794.  Column pass (lane =
// column k2): the 32-point inverse transform over k1 as two 16-point
// transforms of the even and odd rows, Y[n] = E[n mod 16] + w32^n O[n mod 16]
// (w32^(n + 16) = -w32^n), evaluated for the 16 kept rows n = o .. o + 15
// only; they go to shared memory.  Row pass: lane 2r + h takes kept row r and
// the outputs n2 = 2m + h: Out[2m + h] = DFT16_m[(z[k] + (-1)^h z[k + 16])
// w32^(k h)], of which the 8 kept ones (n2 in o .. o + 15) are stored.
template <int S>
__global__ void __launch_bounds__(256, 3) k_aw_fftconv_f(
    const float2 *__restrict__ fa, const float2 *__restrict__ fw, int nW, int QQ,
    const int32_t *__restrict__ wi, float2 *__restrict__ out, int32_t *status) {
  using f32::cf;
  __shared__ float2 sfa[32][33];
  __shared__ float2 srow[8][16][33];  // per warp: the kept rows of the column pass
  constexpr int o = (S - 1) / 2;
  const int k = blockIdx.x;
  const int w = wi[k];
  if (w < 0 || w >= nW) {
    if (threadIdx.x == 0) atomicAdd(&status[ST_INDEX], 1);
    return;
  }
  if ((status[ST_RANGE] | status[ST_INDEX]) != 0) return;
  for (int t = threadIdx.x; t < 1024; t += blockDim.x)
    sfa[t >> 5][t & 31] = fa[(int64_t)k * 1024 + t];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int r = lane >> 1, h = lane & 1;
  auto mul = [](cf a, float2 b) { return cf{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; };
  for (int f = warp; f < QQ; f += 8) {
    const float2 *src = fw + ((int64_t)w * QQ + f) * 1024;
    cf e[16], od[16];
#pragma unroll
    for (int b = 0; b < 16; ++b) {
      const float2 x0 = src[(2 * b) * 32 + lane], a0 = sfa[2 * b][lane];
      const float2 x1 = src[(2 * b + 1) * 32 + lane], a1 = sfa[2 * b + 1][lane];
      e[b] = mul(cf{a0.x, a0.y}, x0);
      od[b] = mul(cf{a1.x, a1.y}, x1);
    }
    f32::dft16(e, 1);  // inverse: exp(+2 pi i / 16); output q in slot out_slot(4, q)
    f32::dft16(od, 1);
#pragma unroll
    for (int t = 0; t < 16; ++t) {
      const int n = o + t, q = n < 16 ? n : n - 16;
      const cf E = e[f32::out_slot(4, q)], O = mul(od[f32::out_slot(4, q)], c_tw32[q]);
      const cf y = n < 16 ? f32::cf_add(E, O) : f32::cf_sub(E, O);
      srow[warp][t][lane] = make_float2(y.x, y.y);
    }
    __syncwarp();
    cf u[16];
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      const float2 z0 = srow[warp][r][kk], z1 = srow[warp][r][kk + 16];
      const cf sum = {z0.x + z1.x, z0.y + z1.y}, dif = {z0.x - z1.x, z0.y - z1.y};
      u[kk] = h ? mul(dif, c_tw32[kk]) : sum;
    }
    __syncwarp();  // srow is rewritten by the next sub-kernel
    f32::dft16(u, 1);
    float2 *dst = out + ((int64_t)k * QQ + f) * 256 + r * 16;
    constexpr int m0e = (o + 1) >> 1, m0o = o >> 1;  // first kept m for h = 0 and 1
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int me = m0e + j, mo = m0o + j;  // n2 = 2 me, or 2 mo + 1
      const cf v = h ? u[f32::out_slot(4, mo)] : u[f32::out_slot(4, me)];
      dst[(h ? 2 * mo + 1 : 2 * me) - o] = make_float2(v.x, v.y);
    }
  }
}

}  // namespace

bool aw_fft_supported(int SA, int S) { return SA == 16 && S >= 1 && S <= 16; }

// room for either precision (complex128 spectra)
size_t aw_fft_workspace_bytes(int nk, int nW, int Q) {
  return ((size_t)std::max(nk, 1) + (size_t)std::max(nW, 1) * Q * Q) * 1024 * sizeof(double2);
}

namespace {

// akern: [nk][16][16] A1 (*) A2 kernels in precision R, W: [nW][Q][Q][S][S] FP64;
// out: [nk][Q][Q][16][16] complex64 (R = float) or complex128 (R = double).
template <typename R>
int aw_fft_run(const typename Cx<R>::T *akern, int nk, const void *W, int nW, int Q, int S,
               const int32_t *wi, void *out, void *ws, size_t ws_bytes, int32_t *d_status,
               cudaStream_t st) {
  typedef typename Cx<R>::T T;
  CG_REQUIRE(aw_fft_supported(16, S), "FFT AW convolution needs 16 x 16 kernels, S <= 16");
  if (ws_bytes < aw_fft_workspace_bytes(nk, nW, Q))
    return set_error(CG_ERR_WORKSPACE, "AW FFT convolution workspace too small");
  T tw[32];
  for (int t = 0; t < 32; ++t) {
    tw[t].x = (R)std::cos(2.0 * M_PI * t / 32.0);
    tw[t].y = (R)std::sin(2.0 * M_PI * t / 32.0);
  }
  if (sizeof(R) == 4)
    CG_CUDA(cudaMemcpyToSymbolAsync(c_tw32, tw, sizeof(tw), 0, cudaMemcpyHostToDevice, st));
  else
    CG_CUDA(cudaMemcpyToSymbolAsync(c_tw32d, tw, sizeof(tw), 0, cudaMemcpyHostToDevice, st));
  T *fa = (T *)ws;
  T *fw = fa + (size_t)nk * 1024;
  const int64_t nwq = (int64_t)nW * Q * Q;
  const unsigned gb = (unsigned)std::min<int64_t>(((int64_t)nk * 1024 + 255) / 256,
                                                  (int64_t)num_sms() * 16);
  k_pad_akern<T><<<gb, 256, 0, st>>>(akern, nk, fa);
  CG_LAUNCH("AW FFT pad A");
  const unsigned gw = (unsigned)std::min<int64_t>((nwq * 1024 + 255) / 256,
                                                  (int64_t)num_sms() * 16);
  k_pad_w<T><<<gw, 256, 0, st>>>((const double2 *)W, nwq, S, fw);
  CG_LAUNCH("AW FFT pad W");
  cufftHandle plan;
  int rc;
  for (int pass = 0; pass < 2; ++pass) {
    const int batch = pass ? (int)nwq : nk;
    T *data = pass ? fw : fa;
    if ((rc = fft_plan(batch, 32, 32, sizeof(R) == 4 ? CUFFT_C2C : CUFFT_Z2Z, &plan))) return rc;
    if (cufftSetStream(plan, st) != CUFFT_SUCCESS)
      return set_error(CG_ERR_CUDA, "cufftSetStream failed");
    const cufftResult r =
        sizeof(R) == 4
            ? cufftExecC2C(plan, (cufftComplex *)data, (cufftComplex *)data, CUFFT_FORWARD)
            : cufftExecZ2Z(plan, (cufftDoubleComplex *)data, (cufftDoubleComplex *)data,
                           CUFFT_FORWARD);
    if (r != CUFFT_SUCCESS)
      return set_error(CG_ERR_CUDA, "cuFFT failed (AW FFT convolution)");
  }
  const int QQ = Q * Q;
#define CG_AW_FFT_CASE(SS)                                                                 \
  case SS:                                                                                 \
    if constexpr (sizeof(R) == 4)                                                          \
      k_aw_fftconv_f<SS><<<nk, 256, 0, st>>>(fa, fw, nW, QQ, wi, (float2 *)out, d_status);  \
    else                                                                                   \
      k_aw_fftconv<T, SS><<<nk, 256, 0, st>>>(fa, fw, nW, QQ, wi, (T *)out, d_status);     \
    break;
  switch (S) {
    CG_AW_FFT_CASE(1) CG_AW_FFT_CASE(2) CG_AW_FFT_CASE(3) CG_AW_FFT_CASE(4)
    CG_AW_FFT_CASE(5) CG_AW_FFT_CASE(6) CG_AW_FFT_CASE(7) CG_AW_FFT_CASE(8)
    CG_AW_FFT_CASE(9) CG_AW_FFT_CASE(10) CG_AW_FFT_CASE(11) CG_AW_FFT_CASE(12)
    CG_AW_FFT_CASE(13) CG_AW_FFT_CASE(14) CG_AW_FFT_CASE(15) CG_AW_FFT_CASE(16)
  }
#undef CG_AW_FFT_CASE
  CG_LAUNCH("AW FFT convolution");
  return CG_OK;
}

}  // namespace

int aw_fft_launch(const float2 *akern, int nk, const void *W, int nW, int Q, int S,
                  const int32_t *wi, void *out, int out_c64, void *ws, size_t ws_bytes,
                  int32_t *d_status, cudaStream_t st) {
  CG_REQUIRE(out_c64, "aw_fft_launch writes complex64 tables");
  return aw_fft_run<float>(akern, nk, W, nW, Q, S, wi, out, ws, ws_bytes, d_status, st);
}

// complex128 tables in FP64 throughout: FP64 spectra, products and transforms
int aw_fft_launch64(const double2 *akern, int nk, const void *W, int nW, int Q, int S,
                    const int32_t *wi, void *out, void *ws, size_t ws_bytes, int32_t *d_status,
                    cudaStream_t st) {
  return aw_fft_run<double>(akern, nk, W, nW, Q, S, wi, out, ws, ws_bytes, d_status, st);
}

}  // namespace cg
