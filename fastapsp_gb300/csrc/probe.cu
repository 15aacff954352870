// probe.cu -- add-min issue-rate microbenchmark (the roofline denominator of
// the Floyd-Warshall and min-plus phases; no counterpart in the reference).
//
// Each thread keeps 64 independent accumulators (32 for the forms that keep
// an index beside each value) and applies the add-min operation of the
// chosen kind to them from register operands only (no memory traffic), so
// the kernel runs at the SM's issue limit for that instruction sequence.
// Operands rotate over 4 register sets and one set is bumped per pass so
// that the compiler cannot fold repeated minima; the bump costs one
// instruction per 16 add-mins, which makes the measured peak a slight
// underestimate.
//   mode 0: int32 DPX add-min   acc = __viaddmin_u32(a, b, acc)
//   mode 1: FP32 add-min        acc = fminf(a + b, acc)
//   mode 2: int32 add-min keeping the argmin (the tile kernel's inner step)
//   mode 3: FP32 add-min keeping the argmin
//   mode 4: int32, two add-mins per step: two adds and one 3-input min (DPX)
//   mode 5: FP32, two add-mins per step: one paired add (add.f32x2) and one
//           3-input min
//   modes 6-9: FP32 add-min keeping the step index of the last strict
//           improvement (the FP32 strip kernel's step), written four ways:
//           6 __vibmin_s32 (values are non-negative floats), 7 one unsigned
//           compare and two predicated moves, 8 a float compare, fminf and a
//           select, 9 __vibmin_u32 (the single-step form of the FP32
//           kernels)
//   mode 10: FP32 add-mins in groups of four steps keeping the group of the
//           last strict improvement: four adds, a 3-input and a 2-input
//           minimum, one compare, two selects
//   mode 11: mode 10 with the four adds as two paired adds (add.f32x2) on
//           operands held as step pairs
//   mode 12: the groups of four as the FP32 strip kernels run them: four
//           adds, two 3-input minimums with the current value as an input,
//           one compare, one select

#include <cuda_runtime.h>
#include <stdint.h>

#include "launch.h"

namespace fapk {

namespace {

__device__ __forceinline__ unsigned min3_u32(unsigned a, unsigned b, unsigned c) {
  return __vimin3_u32(a, b, c);
}
__device__ __forceinline__ float min3_f32(float a, float b, float c) {
  float d;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
__device__ __forceinline__ float2 add_f32x2(float2 a, float2 b) {
  unsigned long long x, y, z;
  x = (unsigned long long)__float_as_uint(a.x) | ((unsigned long long)__float_as_uint(a.y) << 32);
  y = (unsigned long long)__float_as_uint(b.x) | ((unsigned long long)__float_as_uint(b.y) << 32);
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(z) : "l"(x), "l"(y));
  return make_float2(__uint_as_float((unsigned)z), __uint_as_float((unsigned)(z >> 32)));
}

// Output columns per thread (4 rows each): 16, or 8 for the forms that keep
// an index beside each value, so that the outputs and operands stay in
// registers.
__host__ __device__ constexpr int probe_cols(int mode) { return mode == 2 || mode == 3 || mode >= 6 ? 8 : 16; }

template <int MODE>
__global__ void __launch_bounds__(256) addmin_peak_kernel(unsigned *out, int iters, unsigned seed) {
  constexpr bool F = (MODE == 1 || MODE == 3 || MODE == 5 || MODE >= 6);
  constexpr bool GROUPED = MODE >= 10;
  constexpr bool ARG = (MODE == 2 || MODE == 3 || MODE >= 6);
  using T = typename std::conditional<F, float, unsigned>::type;
  constexpr int NC = probe_cols(MODE);
  T a[4][4], b[4][NC], acc[4][NC];
  int arg[4][NC];
  const unsigned t = threadIdx.x + blockIdx.x * blockDim.x + seed;
#pragma unroll
  for (int s = 0; s < 4; s++)
#pragma unroll
    for (int i = 0; i < NC; i++) {
      if (i < 4) a[s][i] = (T)((t * 7 + s * 13 + i * 3) & 1023);
      b[s][i] = (T)((t * 5 + s * 11 + i * 17) & 1023);
    }
#pragma unroll
  for (int r = 0; r < 4; r++)
#pragma unroll
    for (int c = 0; c < NC; c++) {
      acc[r][c] = (T)(1 << 20);
      arg[r][c] = 0;
    }
  // four passes per trip, so that the bumped register set has a fixed index
  // (a register-array index that varies at run time puts the array in local
  // memory)
  for (int it0 = 0; it0 < iters; it0 += 4)
#pragma unroll
  for (int u = 0; u < 4; u++) {
    const int it = it0 + u;
    if constexpr (GROUPED) {
      const int grp = it * 4 + 1;
#pragma unroll
      for (int r = 0; r < 4; r++)
#pragma unroll
        for (int c = 0; c < NC; c++) {
          unsigned v0, v1, v2, v3;
          if (MODE != 11) {
            v0 = __float_as_uint(__fadd_rn((float)a[0][r], (float)b[0][c]));
            v1 = __float_as_uint(__fadd_rn((float)a[1][r], (float)b[1][c]));
            v2 = __float_as_uint(__fadd_rn((float)a[2][r], (float)b[2][c]));
            v3 = __float_as_uint(__fadd_rn((float)a[3][r], (float)b[3][c]));
          } else {
            const float2 p01 = add_f32x2(make_float2((float)a[0][r], (float)a[1][r]),
                                         make_float2((float)b[0][c], (float)b[1][c]));
            const float2 p23 = add_f32x2(make_float2((float)a[2][r], (float)a[3][r]),
                                         make_float2((float)b[2][c], (float)b[3][c]));
            v0 = __float_as_uint(p01.x), v1 = __float_as_uint(p01.y);
            v2 = __float_as_uint(p23.x), v3 = __float_as_uint(p23.y);
          }
          const unsigned ac = __float_as_uint((float)acc[r][c]);
          if (MODE == 12) {
            const unsigned na = __vimin3_u32(ac, __vimin3_u32(v0, v1, v2), v3);
            arg[r][c] = na != ac ? grp : arg[r][c];
            acc[r][c] = (T)__uint_as_float(na);
          } else {
            const unsigned t = min(__vimin3_u32(v0, v1, v2), v3);
            const bool imp = t < ac;
            acc[r][c] = (T)__uint_as_float(imp ? t : ac);
            arg[r][c] = imp ? grp : arg[r][c];
          }
        }
    } else if constexpr (MODE == 4 || MODE == 5) {
#pragma unroll
      for (int s = 0; s < 4; s += 2)
#pragma unroll
        for (int r = 0; r < 4; r++)
#pragma unroll
          for (int c = 0; c < NC; c++) {
            if (MODE == 4) {
              acc[r][c] = (T)min3_u32((unsigned)acc[r][c], (unsigned)a[s][r] + (unsigned)b[s][c],
                                      (unsigned)a[s + 1][r] + (unsigned)b[s + 1][c]);
            } else {
              const float2 v = add_f32x2(make_float2((float)a[s][r], (float)a[s + 1][r]),
                                         make_float2((float)b[s][c], (float)b[s + 1][c]));
              acc[r][c] = (T)min3_f32((float)acc[r][c], v.x, v.y);
            }
          }
    } else {
#pragma unroll
      for (int s = 0; s < 4; s++) {
#pragma unroll
        for (int r = 0; r < 4; r++)
#pragma unroll
          for (int c = 0; c < NC; c++) {
            const T x = a[s][r], y = b[s][c];
            const int idx = it * 4 + s + 1;
            if (MODE == 0) {
              acc[r][c] = (T)__viaddmin_u32((unsigned)x, (unsigned)y, (unsigned)acc[r][c]);
            } else if (MODE >= 6) {
              const float fv = (float)x + (float)y;
              const unsigned v = __float_as_uint(fv);
              unsigned ac = __float_as_uint((float)acc[r][c]);
              int ag = arg[r][c];
              if (MODE == 6) {
                bool keep;
                ac = (unsigned)__vibmin_s32((int)ac, (int)v, &keep);
                ag = keep ? ag : idx;
              } else if (MODE == 7) {
                asm("{\n\t.reg .pred p;\n\tsetp.lt.u32 p, %2, %0;\n\t@p mov.b32 %0, %2;\n\t@p mov.b32 %1, %3;\n\t}"
                    : "+r"(ac), "+r"(ag)
                    : "r"(v), "r"(idx));
              } else if (MODE == 8) {
                const float fa = __uint_as_float(ac);
                const bool lt = fv < fa;
                ac = __float_as_uint(fminf(fa, fv));
                ag = lt ? idx : ag;
              } else {
                bool keep;
                ac = __vibmin_u32(ac, v, &keep);
                ag = keep ? ag : idx;
              }
              acc[r][c] = (T)__uint_as_float(ac);
              arg[r][c] = ag;
            } else if (MODE == 1) {
              acc[r][c] = fminf((float)x + (float)y, (float)acc[r][c]);
            } else {
              const T v = x + y;
              if (v < acc[r][c]) {
                acc[r][c] = v;
                arg[r][c] = s;
              }
            }
          }
      }
    }
#pragma unroll
    for (int i = 0; i < NC; i++) b[u][i] = b[u][i] - (T)1;
  }
  unsigned x = 0;
#pragma unroll
  for (int r = 0; r < 4; r++)
#pragma unroll
    for (int c = 0; c < NC; c++) {
      unsigned v;
      if (F) v = __float_as_uint((float)acc[r][c]); else v = (unsigned)acc[r][c];
      x ^= v + (ARG ? (unsigned)arg[r][c] : 0u);
    }
  out[threadIdx.x + blockIdx.x * blockDim.x] = x;
}

template <int MODE>
cudaError_t run_mode(unsigned *buf, int blocks, int iters, cudaStream_t st) {
  addmin_peak_kernel<MODE><<<blocks, 256, 0, st>>>(buf, iters, 1u);
  return cudaGetLastError();
}

}  // namespace

// Returns add-min operations per second of `mode` on the current device.
cudaError_t measure_addmin_peak(int mode, int sm_count, double *ops_per_s) {
  const int blocks = sm_count * 8;  // 8 x 256 threads per SM
  const int iters = 2048;
  unsigned *buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, (size_t)blocks * 256 * sizeof(unsigned));
  if (e != cudaSuccess) return e;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best = 1e30f;
  for (int rep = 0; rep < 4; rep++) {
    cudaEventRecord(a, 0);
    switch (mode) {
      case 0: e = run_mode<0>(buf, blocks, iters, 0); break;
      case 1: e = run_mode<1>(buf, blocks, iters, 0); break;
      case 2: e = run_mode<2>(buf, blocks, iters, 0); break;
      case 3: e = run_mode<3>(buf, blocks, iters, 0); break;
      case 4: e = run_mode<4>(buf, blocks, iters, 0); break;
      case 5: e = run_mode<5>(buf, blocks, iters, 0); break;
      case 6: e = run_mode<6>(buf, blocks, iters, 0); break;
      case 7: e = run_mode<7>(buf, blocks, iters, 0); break;
      case 8: e = run_mode<8>(buf, blocks, iters, 0); break;
      case 9: e = run_mode<9>(buf, blocks, iters, 0); break;
      case 10: e = run_mode<10>(buf, blocks, iters, 0); break;
      case 11: e = run_mode<11>(buf, blocks, iters, 0); break;
      default: e = run_mode<12>(buf, blocks, iters, 0); break;
    }
    cudaEventRecord(b, 0);
    if (e != cudaSuccess) break;
    e = cudaEventSynchronize(b);
    if (e != cudaSuccess) break;
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    if (rep > 0) best = ms < best ? ms : best;  // first launch is warm-up
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(buf);
  if (e != cudaSuccess) return e;
  const int cols = probe_cols(mode);
  const double ops = (double)blocks * 256 * iters * 4 * 4 * cols;
  *ops_per_s = ops / (best * 1e-3);
  return cudaSuccess;
}

}  // namespace fapk
