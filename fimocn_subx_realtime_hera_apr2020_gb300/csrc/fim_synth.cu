// Seeded balanced initial state made on the device (fim_state_synthetic).
//
// The reference takes its initial state from GFS data (ss2icos,
// dyn_init.F90:826), which is not in the tree; the seeded state here is the
// same recipe as the package's host generator (state.py): surface pressure
// 1000 hPa + N(0, sigma_ps), layer thicknesses proportional to dpsig,
// potential temperature rising linearly from 300 K to 600 K, zonal wind
// 35 m/s cos(lat) (+ N(0, noise) on u and v), tracers 2..ntra drawn
// U[0, 1e-2), flat topography.  The random numbers come from a counter-based
// generator, so every value depends only on the seed and its position: a
// state is the same whatever the launch shape, the member slot or the
// context it is made in (but not the numbers of the host generator).
//
// Generator: SplitMix64's output function (Steele, Lea and Flood, "Fast
// splittable pseudorandom number generators", OOPSLA 2014) applied to a Weyl
// sequence keyed by (seed, stream); uniforms from the top 53 bits; normals by
// the Box-Muller transform.
#include "fim_internal.h"

namespace fim {

namespace {

constexpr int kSynthBlock = 256;
constexpr unsigned long long kGolden = 0x9E3779B97F4A7C15ull;

__host__ __device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// the idx-th 64-bit value of stream `stream` under `seed`
__device__ __forceinline__ unsigned long long draw(unsigned long long seed, unsigned long long stream,
                                                   unsigned long long idx) {
  const unsigned long long key = mix64(seed * kGolden + stream);
  return mix64(key + (idx + 1) * kGolden);
}

// U[0, 1)
__device__ __forceinline__ double uniform(unsigned long long seed, unsigned long long stream,
                                          unsigned long long idx) {
  return (double)(draw(seed, stream, idx) >> 11) * 0x1.0p-53;
}

// N(0, 1): Box-Muller on two uniforms of the stream, the first in (0, 1]
__device__ __forceinline__ double normal(unsigned long long seed, unsigned long long stream,
                                         unsigned long long idx) {
  const double u1 = (double)((draw(seed, stream, 2 * idx) >> 11) + 1) * 0x1.0p-53;
  const double u2 = (double)(draw(seed, stream, 2 * idx + 1) >> 11) * 0x1.0p-53;
  return sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
}

// streams of the state's random values
enum : unsigned long long { kStreamPs = 1, kStreamU = 2, kStreamV = 3, kStreamTracer = 16 };

// One column a thread: surface pressure, interface pressures summed down
// from the top, layer thicknesses, Exner function, zero geopotential.
template <typename R>
__global__ void __launch_bounds__(kSynthBlock) k_synth_columns(int N, int L, const double* __restrict__ dps,
    unsigned long long seed, double sigma_ps, double ptop, R* __restrict__ dp3d, R* __restrict__ pr3d,
    R* __restrict__ ex3d, R* __restrict__ ph3d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int L1 = L + 1;
  const double ps = kP1000 + normal(seed, kStreamPs, (unsigned long long)i) * sigma_ps;
  R* pr = pr3d + (size_t)i * L1;
  R* ex = ex3d + (size_t)i * L1;
  double above = ptop, acc = 0.0;
  pr[L] = R(ptop);
  ex[L] = R(kCp * pow(ptop / kP1000, kRd / kCp));
  ph3d[(size_t)i * L1 + L] = R(0);
  for (int k = L - 1; k >= 0; k--) {
    acc += (ps - ptop) * dps[k];
    const double p = ptop + acc;
    pr[k] = R(p);
    ex[k] = R(kCp * pow(p / kP1000, kRd / kCp));
    dp3d[(size_t)i * L + k] = R(p - above);
    ph3d[(size_t)i * L1 + k] = R(0);
    above = p;
  }
}

// One cell-level a thread: winds, Montgomery potential (zero: hystat forms
// it) and every tracer slot of the member (theta, the drawn tracers 1..ntra-1,
// zero past ntra).
template <typename R>
__global__ void __launch_bounds__(kSynthBlock) k_synth_levels(int N, int L, int nslot, int ntra,
    const double* __restrict__ lat, unsigned long long seed, double noise, R* __restrict__ us3d,
    R* __restrict__ vs3d, R* __restrict__ mp3d, R* __restrict__ tr3d) {
  const size_t NL = (size_t)N * L;
  const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= NL) return;
  const int i = (int)(c / L), k = (int)(c - (size_t)i * L);
  double u = 35.0 * cos(lat[i]), v = 0.0;
  if (noise > 0.0) {
    u += normal(seed, kStreamU, c) * noise;
    v += normal(seed, kStreamV, c) * noise;
  }
  us3d[c] = R(u);
  vs3d[c] = R(v);
  mp3d[c] = R(0);
  tr3d[c] = R(300.0 + 300.0 * k / (L - 1));
  for (int t = 1; t < nslot; t++)
    tr3d[(size_t)t * NL + c] = t < ntra ? R(uniform(seed, kStreamTracer + t, c) * 1e-2) : R(0);
}

}  // namespace

template <typename R>
int launch_synthetic(cudaStream_t stream, int N, int L, int nslot, int ntra, const double* lat,
                     const double* dps, unsigned long long seed, double sigma_ps, double noise, double ptop,
                     R* us3d, R* vs3d, R* dp3d, R* pr3d, R* ex3d, R* ph3d, R* mp3d, R* tr3d) {
  k_synth_columns<R><<<(unsigned)((N + kSynthBlock - 1) / kSynthBlock), kSynthBlock, 0, stream>>>(
      N, L, dps, seed, sigma_ps, ptop, dp3d, pr3d, ex3d, ph3d);
  const size_t NL = (size_t)N * L;
  k_synth_levels<R><<<(unsigned)((NL + kSynthBlock - 1) / kSynthBlock), kSynthBlock, 0, stream>>>(
      N, L, nslot, ntra, lat, seed, noise, us3d, vs3d, mp3d, tr3d);
  return (int)cudaGetLastError();
}

template int launch_synthetic<float>(cudaStream_t, int, int, int, int, const double*, const double*,
                                     unsigned long long, double, double, double, float*, float*, float*, float*,
                                     float*, float*, float*, float*);
template int launch_synthetic<double>(cudaStream_t, int, int, int, int, const double*, const double*,
                                      unsigned long long, double, double, double, double*, double*, double*,
                                      double*, double*, double*, double*, double*);

}  // namespace fim
