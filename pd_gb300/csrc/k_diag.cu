// k_diag.cu — measurement aids: the FP32 FMA ceiling of this GPU and a census
// of the pairs the pair kernels evaluate, by the branch each takes.  Neither
// has a counterpart in PD; the benchmark's roofline divides exact pair counts
// of each branch, times that branch's flops, by the kernel's time, against the
// measured FMA ceiling.
#include "pdgpu_tile.cuh"

namespace pdgpu {

// ---------------------------------------------------------------------------
// FP32 FMA ceiling: kChains independent FMA chains per thread (FFMA, or FFMA2
// on float2 pairs), enough warps per scheduler to cover the FMA latency.  The
// result is written so the chains are not removed.
// ---------------------------------------------------------------------------
constexpr int kChains = 8;

template <bool PACKED>
__global__ void __launch_bounds__(256) k_fma_probe(float* out, int iters, float b, float c) {
  float s = 0.f;
  if (PACKED) {
    float2 a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; k++) a[k] = make_float2(threadIdx.x * 1e-3f + k, blockIdx.x * 1e-3f - k);
    const float2 B = make_float2(b, b), C = make_float2(c, c);
    for (int it = 0; it < iters; it++) {
#pragma unroll
      for (int k = 0; k < kChains; k++) a[k] = __ffma2_rn(a[k], B, C);
    }
#pragma unroll
    for (int k = 0; k < kChains; k++) s += a[k].x + a[k].y;
  } else {
    float a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; k++) a[k] = threadIdx.x * 1e-3f + blockIdx.x * 1e-3f + k;
    for (int it = 0; it < iters; it++) {
#pragma unroll
      for (int k = 0; k < kChains; k++) a[k] = fmaf(a[k], b, c);
    }
#pragma unroll
    for (int k = 0; k < kChains; k++) s += a[k];
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// ---------------------------------------------------------------------------
// Pair census over the current tile list (one warp per tile, the j block
// rotated by shuffles as in the pair kernels), FP32 decisions as the kernels
// take them:
//   [0] FF_NonBonded pairs inside Cutoff (bond order > 2)
//   [1] GB pairs inside the GB Cutoff (every pair, as calcForcesIncludingVacuo)
//   [2]   of which above ExpApproxThreshold (the GB cross term is evaluated)
//   [3] Born-radius pairs inside GbsaStillCutoff (bond order > 2)
//   [4]   of which in close contact (the CCF branch)
// The GB counts use the Born radii of the last GB evaluation.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float gb_u_census(float r2, float ai, float aj) { return -0.25f * __fdividef(r2, ai * aj); }

__global__ void __launch_bounds__(256) k_census(const __grid_constant__ DevView v, const __grid_constant__ NBConst nk, const __grid_constant__ GBConst gk, int do_nb, int do_gb,
                                                const float* born, unsigned long long* out) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nt = *v.ntiles;
  unsigned long long c[5] = {0, 0, 0, 0, 0};
  for (int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < nt; t += nwarps) {
    const Tile T = v.tiles[t];
    const SystemInfo& S = v.sys[v.slot_sys[T.bi]];
    const int si = T.bi * 32 + lane;
    const float4 xi = v.xq[si], pi = v.par[si];
    const float ai = born ? born[si] : 1.f;
    unsigned ex, m14;
    tile_masks(v, T, lane, ex, m14);
    const unsigned dmask = (T.flags & 2) ? diag_exclusion(lane) : 0u;
    float4 xj = j_in_i_frame(v, T, lane);
    float4 pj = v.par[T.bj * 32 + lane];
    float aj = born ? born[T.bj * 32 + lane] : 1.f;
    const bool mi = (T.flags & 1) && S.periodic;
    for (int kk = 0; kk < 32; kk++) {
      float dx = xj.x - xi.x, dy = xj.y - xi.y, dz = xj.z - xi.z;
      if (mi) {
        dx -= (float)S.box[0] * rintf(dx * (float)S.ibox[0]);
        dy -= (float)S.box[1] * rintf(dy * (float)S.ibox[1]);
        dz -= (float)S.box[2] * rintf(dz * (float)S.ibox[2]);
      }
      const float r2 = dx * dx + dy * dy + dz * dz;
      const bool pair = !((dmask >> kk) & 1u);
      const bool bonded_out = (ex >> kk) & 1u;  // bond order <= 2 (diagonal self pairs included)
      if (do_nb && pair && !bonded_out && r2 <= nk.cut2) c[0]++;
      if (do_gb && pair) {
        if (r2 <= gk.cut2) {
          c[1]++;
          if (gb_u_census(r2, ai, aj) > gk.thresh) c[2]++;
        }
        if (!bonded_out && r2 <= gk.still2) {
          c[3]++;
          const float rs = pi.z + pj.z;
          if (r2 <= rs * rs * gk.invP5) c[4]++;
        }
      }
      ROT(xj.x); ROT(xj.y); ROT(xj.z); ROT(pj.z); ROT(aj);
    }
  }
#pragma unroll
  for (int k = 0; k < 5; k++) {
    unsigned long long x = c[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0 && x) atomicAdd(&out[k], x);
  }
}

int launch_census(Context& c, const NBConst& nk, const GBConst& gk, bool do_nb, bool do_gb, unsigned long long* out) {
  c.kernel_launches += 1;
  k_census<<<tile_grid(c), 256, 0, c.stream>>>(c.view(), nk, gk, do_nb ? 1 : 0, do_gb ? 1 : 0,
                                               do_gb ? c.d_born_f.p : nullptr, out);
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

int measure_fp32_peak(int device, double* tflops_ffma, double* tflops_ffma2) {
  if (cudaSetDevice(device) != cudaSuccess) return PDGPU_ERR_CUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return PDGPU_ERR_CUDA;
  const int blocks = sms * 4, threads = 256, iters = 1 << 14;
  DBuf<float> out;
  if (out.alloc((size_t)blocks * threads) != cudaSuccess) return PDGPU_ERR_CUDA;
  cudaStream_t st;
  cudaEvent_t e0, e1;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return PDGPU_ERR_CUDA;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best[2] = {1e30, 1e30};
  for (int packed = 0; packed < 2; packed++) {
    for (int rep = 0; rep < 6; rep++) {  // the first launch warms up and is not counted
      cudaEventRecord(e0, st);
      if (packed) k_fma_probe<true><<<blocks, threads, 0, st>>>(out.p, iters, 0.999999f, 1e-6f);
      else k_fma_probe<false><<<blocks, threads, 0, st>>>(out.p, iters, 0.999999f, 1e-6f);
      cudaEventRecord(e1, st);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0 && ms < best[packed]) best[packed] = ms;
    }
  }
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(st);
  if (err != cudaSuccess) return PDGPU_ERR_CUDA;
  const double fmas = (double)blocks * threads * iters * kChains;  // per launch (FFMA2 does two per chain step)
  if (tflops_ffma) *tflops_ffma = 2.0 * fmas / (best[0] * 1e-3) / 1e12;
  if (tflops_ffma2) *tflops_ffma2 = 4.0 * fmas / (best[1] * 1e-3) / 1e12;
  return PDGPU_OK;
}

}  // namespace pdgpu
