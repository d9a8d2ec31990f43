// k_selftest.cu -- on-device self-tests of the tensor-core building blocks.
//
// rpa_selftest(RPA_SELFTEST_UMMA, ...) runs one 128 x N x K bf16 GEMM with
// tcgen05.mma out of 128-byte-swizzled shared-memory tiles into a TMEM
// accumulator and compares it with an FP32 CUDA-core dot product of the same
// bf16 values.  It checks the descriptor encodings, the swizzle layout and
// the TMEM read-back before the accumulation kernels rely on them.

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "rpa_internal.cuh"
#include "tc05.cuh"

namespace rpa {

__device__ __forceinline__ float hval(uint32_t a, uint32_t b, uint32_t seed) {
  uint32_t h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u) * 0x85EBCA77u ^ seed * 0xC2B2AE3Du;
  h ^= h >> 15;
  h *= 0x2C1B3C6Du;
  h ^= h >> 12;
  return (float)(h & 0xFFFF) / 32768.0f - 1.0f;
}

template <int N>
__global__ void __launch_bounds__(128) k_umma_selftest(int nchunks, uint32_t seed, float* out, float* ref,
                                                       int* status) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(sm) + 1023) & ~uintptr_t(1023));
  unsigned char* A = base;                 // 128 x 128 B
  unsigned char* B = base + 128 * 128;     // N x 128 B
  __shared__ uint64_t bar;
  __shared__ uint32_t tslot;
  constexpr uint32_t NCOL = N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : (N <= 256 ? 256 : 512)));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) {
    tc::tmem_alloc(&tslot, NCOL);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t taddr = tslot;
  bool ok = true;
  for (int c = 0; c < nchunks && ok; ++c) {
    for (int e = tid; e < 128 * 64; e += 128) {
      int r = e >> 6, k = e & 63;
      *reinterpret_cast<__nv_bfloat16*>(A + tc::sw128_off(r, k)) = __float2bfloat16_rn(hval(r, c * 64 + k, seed));
    }
    for (int e = tid; e < N * 64; e += 128) {
      int r = e >> 6, k = e & 63;
      *reinterpret_cast<__nv_bfloat16*>(B + tc::sw128_off(r, k)) =
          __float2bfloat16_rn(hval(1000 + r, c * 64 + k, seed));
    }
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::tc_fence_after();
      const uint32_t idesc = tc::idesc_bf16(128, N);
#pragma unroll
      for (int ks = 0; ks < 4; ++ks)
        tc::mma_bf16(taddr, tc::desc_sw128(tc::smem_u32(A) + ks * 32), tc::desc_sw128(tc::smem_u32(B) + ks * 32),
                     idesc, (c > 0 || ks > 0) ? 1u : 0u);
      tc::mma_commit(&bar);
    }
    ok = tc::mbar_wait(&bar, c & 1, 1u << 16);
    if (!ok) atomicExch(status, 1);
    tc::tc_fence_after();
    __syncthreads();
  }
  if (ok) {
    for (int c0 = 0; c0 < N; c0 += 32) {
      float v[32];
      tc::tmem_ld32(taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      tc::tmem_ld_wait();
      int row = warp * 32 + lane;
#pragma unroll
      for (int i = 0; i < 32; ++i)
        if (c0 + i < N) out[row * N + c0 + i] = v[i];
    }
  }
  // CUDA-core reference of the same bf16 products
  for (int e = tid; e < 128 * N; e += 128) {
    int r = e / N, n = e % N;
    float s = 0.f;
    for (int k = 0; k < nchunks * 64; ++k)
      s += __bfloat162float(__float2bfloat16_rn(hval(r, k, seed))) *
           __bfloat162float(__float2bfloat16_rn(hval(1000 + n, k, seed)));
    ref[e] = s;
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, NCOL);
}

int selftest_umma(int which, double* result) {
  // which: 0 -> N=192, 1 -> N=96, 2 -> N=256
  int N = which == 1 ? 96 : (which == 2 ? 256 : 192);
  const int nchunks = 3;
  float *out = nullptr, *ref = nullptr;
  int* status = nullptr;
  size_t n = (size_t)128 * N;
  if (cudaMalloc(&out, n * 4) != cudaSuccess || cudaMalloc(&ref, n * 4) != cudaSuccess ||
      cudaMalloc(&status, 4) != cudaSuccess)
    return RPA_ENOMEM;
  cudaMemset(out, 0, n * 4);
  cudaMemset(status, 0, 4);
  size_t smem = 1024 + 128 * 128 + (size_t)N * 128;
  cudaError_t e;
  if (N == 192) {
    cudaFuncSetAttribute(k_umma_selftest<192>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_umma_selftest<192><<<1, 128, smem>>>(nchunks, 12345u, out, ref, status);
  } else if (N == 96) {
    cudaFuncSetAttribute(k_umma_selftest<96>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_umma_selftest<96><<<1, 128, smem>>>(nchunks, 12345u, out, ref, status);
  } else {
    cudaFuncSetAttribute(k_umma_selftest<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_umma_selftest<256><<<1, 128, smem>>>(nchunks, 12345u, out, ref, status);
  }
  e = cudaDeviceSynchronize();
  std::vector<float> ho(n), hr(n);
  int st = 0;
  if (e == cudaSuccess) {
    cudaMemcpy(ho.data(), out, n * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(hr.data(), ref, n * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(&st, status, 4, cudaMemcpyDeviceToHost);
  }
  cudaFree(out);
  cudaFree(ref);
  cudaFree(status);
  if (e != cudaSuccess) return RPA_ECUDA;
  if (st) return RPA_ETIMEOUT;
  double mx = 0, mref = 0;
  for (size_t i = 0; i < n; ++i) {
    mx = std::max(mx, (double)std::fabs(ho[i] - hr[i]));
    mref = std::max(mref, (double)std::fabs(hr[i]));
  }
  *result = mref > 0 ? mx / mref : mx;
  return RPA_OK;
}

// The same GEMM with A in tensor memory (tcgen05.mma with an [a_tmem]
// operand, kind::f16 with f16 inputs): each warp writes the rows of its lane
// quadrant, two f16 of K per 32-bit column (K = 64 per chunk: 32 columns);
// B stays a 128-byte-swizzled K-major tile in shared memory.  Checks the A
// layout in TMEM before a kernel relies on it.
template <int N>
__global__ void __launch_bounds__(128) k_umma_ts_selftest(int nchunks, uint32_t seed, float* out, float* ref,
                                                          int* status) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(sm) + 1023) & ~uintptr_t(1023));
  unsigned char* B = base;  // N x 128 B
  __shared__ uint64_t bar;
  __shared__ uint32_t tslot;
  constexpr uint32_t NCOL = N + 32 <= 64 ? 64 : (N + 32 <= 128 ? 128 : (N + 32 <= 256 ? 256 : 512));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) {
    tc::tmem_alloc(&tslot, NCOL);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t taddr = tslot;
  const uint32_t acol = (uint32_t)N;  // A columns follow the accumulator
  bool ok = true;
  const int row = warp * 32 + lane;
  for (int c = 0; c < nchunks && ok; ++c) {
    // A row `row`: K values c*64 .. c*64+63, packed two per column
#pragma unroll
    for (int g = 0; g < 4; ++g) {
      uint32_t v[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int k = g * 16 + 2 * i;
        const __half2 h = __floats2half2_rn(hval(row, c * 64 + k, seed), hval(row, c * 64 + k + 1, seed));
        v[i] = *reinterpret_cast<const uint32_t*>(&h);
      }
      tc::tmem_st8(taddr + ((uint32_t)(warp * 32) << 16) + acol + (uint32_t)(g * 8), v);
    }
    tc::tmem_st_wait();
    for (int e = tid; e < N * 64; e += 128) {
      int r = e >> 6, k = e & 63;
      *reinterpret_cast<__half*>(B + tc::sw128_off(r, k)) = __float2half_rn(hval(1000 + r, c * 64 + k, seed));
    }
    tc::fence_async_smem();
    tc::tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      tc::tc_fence_after();
      const uint32_t idesc = tc::idesc_bf16(128, N, true);
#pragma unroll
      for (int ks = 0; ks < 4; ++ks)
        tc::mma_ts(taddr, taddr + acol + (uint32_t)(ks * 8), tc::desc_sw128(tc::smem_u32(B) + ks * 32), idesc,
                   (c > 0 || ks > 0) ? 1u : 0u);
      tc::mma_commit(&bar);
    }
    ok = tc::mbar_wait(&bar, c & 1, 1u << 16);
    if (!ok) atomicExch(status, 1);
    tc::tc_fence_after();
    __syncthreads();
  }
  if (ok) {
    for (int c0 = 0; c0 < N; c0 += 32) {
      float v[32];
      tc::tmem_ld32(taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      tc::tmem_ld_wait();
#pragma unroll
      for (int i = 0; i < 32; ++i)
        if (c0 + i < N) out[row * N + c0 + i] = v[i];
    }
  }
  for (int e = tid; e < 128 * N; e += 128) {
    int r = e / N, n = e % N;
    float s = 0.f;
    for (int k = 0; k < nchunks * 64; ++k)
      s += __half2float(__float2half_rn(hval(r, k, seed))) * __half2float(__float2half_rn(hval(1000 + n, k, seed)));
    ref[e] = s;
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, NCOL);
}

int selftest_umma_ts(double* result) {
  constexpr int N = 192;
  const int nchunks = 3;
  float *out = nullptr, *ref = nullptr;
  int* status = nullptr;
  size_t n = (size_t)128 * N;
  if (cudaMalloc(&out, n * 4) != cudaSuccess || cudaMalloc(&ref, n * 4) != cudaSuccess ||
      cudaMalloc(&status, 4) != cudaSuccess)
    return RPA_ENOMEM;
  cudaMemset(out, 0, n * 4);
  cudaMemset(status, 0, 4);
  size_t smem = 1024 + (size_t)N * 128;
  cudaFuncSetAttribute(k_umma_ts_selftest<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_umma_ts_selftest<N><<<1, 128, smem>>>(nchunks, 4321u, out, ref, status);
  cudaError_t e = cudaDeviceSynchronize();
  std::vector<float> ho(n), hr(n);
  int st = 0;
  if (e == cudaSuccess) {
    cudaMemcpy(ho.data(), out, n * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(hr.data(), ref, n * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(&st, status, 4, cudaMemcpyDeviceToHost);
  }
  cudaFree(out);
  cudaFree(ref);
  cudaFree(status);
  if (e != cudaSuccess) return RPA_ECUDA;
  if (st) return RPA_ETIMEOUT;
  double mx = 0, mref = 0;
  for (size_t i = 0; i < n; ++i) {
    mx = std::max(mx, (double)std::fabs(ho[i] - hr[i]));
    mref = std::max(mref, (double)std::fabs(hr[i]));
  }
  *result = mref > 0 ? mx / mref : mx;
  return RPA_OK;
}

// A wait on an mbarrier that nothing arrives on: the bounded wait gives up
// after `polls` suspending polls and the kernel records it in *status and
// returns, the way every wait of the production kernels ends.
__global__ void k_wait_selftest(uint32_t polls, int* status, long long* cycles) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
  }
  __syncthreads();
  const long long t0 = clock64();
  const bool ok = tc::mbar_wait(&bar, 0u, polls);
  if (threadIdx.x == 0) {
    *status = ok ? 0 : 1;
    *cycles = clock64() - t0;
  }
}

// Runs k_wait_selftest; *result = the cycles the wait took.  RPA_ETIMEOUT when
// it gave up (the expected outcome), RPA_OK if it was released.
int selftest_wait(double* result) {
  int* status = nullptr;
  long long* cycles = nullptr;
  if (cudaMalloc(&status, 4) != cudaSuccess || cudaMalloc(&cycles, 8) != cudaSuccess) return RPA_ENOMEM;
  cudaMemset(status, 0, 4);
  k_wait_selftest<<<1, 32>>>(256u, status, cycles);
  cudaError_t e = cudaDeviceSynchronize();
  int st = 0;
  long long cyc = 0;
  if (e == cudaSuccess) {
    cudaMemcpy(&st, status, 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(&cyc, cycles, 8, cudaMemcpyDeviceToHost);
  }
  cudaFree(status);
  cudaFree(cycles);
  if (e != cudaSuccess) return RPA_ECUDA;
  *result = (double)cyc;
  return st ? RPA_ETIMEOUT : RPA_OK;
}

}  // namespace rpa
