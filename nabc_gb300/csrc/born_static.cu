// sffg_born_radii_static(): effective Born radii of one molecule computed
// entirely inside a fixed, statically sized device array.  It allocates
// nothing: no cudaMalloc/cudaFree, no allocating library routine, no host
// heap.
//
// Some callers cannot allocate: a host that hands all device memory to its
// own pool or budget (an extra cudaMalloc can fail or fragment it), or a
// loop that must not stall (cudaFree synchronises the whole device).  They
// use this entry point instead of building a batch, whose set-up allocates
// its device state.
//
// The computation is pass 1 of the reference's egb() followed by its
// radius formula (src/sff/eff.c:1566-1733) with every pair listed, as the
// reference does when cut exceeds the molecule's extent: the descreening
// integral of each ordered pair in FP32, summed per 32-atom tile pair and
// converted to 64-bit fixed point (2^-40), and the HCT / OBC radius of
// every atom in FP64.  It is the batch path's Born-radius step restated for
// a caller-owned molecule: same descreening functions, same fixed-point
// scale, same offset and OBC constants (src/sff/sff.c:1186-1333).
//
// Scratch: one file-scope __device__ array per device, kStaticMaxAtoms
// atoms x 104 bytes (about 0.85 MB).  Every call looks up its device
// address for the current device with cudaGetSymbolAddress (a lookup that
// allocates nothing; the first call on a device also loads this file's
// device code there) and only that address is handed to the kernels, so a
// context that was reset and recreated is picked up.
#include <cuda_runtime.h>

#include <cstdint>

#include "gbmath.cuh"
#include "../../include/sffg.h"

namespace sffg {
namespace {

constexpr int kStaticMaxAtoms = SFFG_STATIC_MAX_ATOMS;
constexpr int kStaticMaxTiles = kStaticMaxAtoms / 32;
constexpr unsigned kAll = 0xffffffffu;

// Byte offsets of the scratch regions (each a multiple of 256).
constexpr size_t kOffX = 0;                                             // double[3N] coordinates
constexpr size_t kOffRb = kOffX + 3 * sizeof(double) * kStaticMaxAtoms;  // double[N] rborn
constexpr size_t kOffFs = kOffRb + sizeof(double) * kStaticMaxAtoms;     // double[N] fs
constexpr size_t kOffHi = kOffFs + sizeof(double) * kStaticMaxAtoms;     // float4[N] x,y,z high parts
constexpr size_t kOffLo = kOffHi + sizeof(float4) * kStaticMaxAtoms;     // float4[N] x,y,z low parts
constexpr size_t kOffGb = kOffLo + sizeof(float4) * kStaticMaxAtoms;     // float4[N] rho, s, rborn, s-correction
constexpr size_t kOffSum = kOffGb + sizeof(float4) * kStaticMaxAtoms;    // int64[N] descreening sums
constexpr size_t kOffReff = kOffSum + sizeof(long long) * kStaticMaxAtoms;  // double[N] radii
constexpr size_t kOffBox = kOffReff + sizeof(double) * kStaticMaxAtoms;  // float4[2T] tile boxes
constexpr size_t kScratchBytes = kOffBox + 2 * sizeof(float4) * kStaticMaxTiles;
static_assert(kStaticMaxAtoms % 32 == 0, "the atom limit must be whole tiles");

__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr double kSumScale = 1099511627776.0;  // 2^40, as the batch path's Born sums

struct StaticArgs {
  unsigned char *base;
  int natom, ntile, gb;
  double offset;
  BornConst born;
};

template <class T>
__device__ __forceinline__ T *region(const StaticArgs &a, size_t off) {
  return reinterpret_cast<T *>(a.base + off);
}

// Splits coordinates into FP32 high + low parts, derives the per-atom
// descreening parameters, clears the sums and records each tile's bounding
// box.  Slots past natom become far-away padding atoms.
__global__ void k_static_pack(const StaticArgs a) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  if (slot - lane >= a.natom) return;  // whole warp past the last tile
  const double *x = region<double>(a, kOffX);
  float4 hi, lo, gp;
  float b0x = 3e38f, b0y = 3e38f, b0z = 3e38f, b1x = -3e38f, b1y = -3e38f, b1z = -3e38f;
  if (slot < a.natom) {
    const double X = x[3 * slot], Y = x[3 * slot + 1], Z = x[3 * slot + 2];
    const float hx = static_cast<float>(X), hy = static_cast<float>(Y), hz = static_cast<float>(Z);
    hi = make_float4(hx, hy, hz, 0.f);
    lo = make_float4(static_cast<float>(X - hx), static_cast<float>(Y - hy), static_cast<float>(Z - hz), 0.f);
    const double rb = region<double>(a, kOffRb)[slot];
    const double rho = rb - a.offset, sd = region<double>(a, kOffFs)[slot] * rho;
    const float sf = static_cast<float>(sd);
    const float scorr = sf != 0.0f ? static_cast<float>(3.0 * (sd - static_cast<double>(sf)) / sf) : 0.0f;
    gp = make_float4(static_cast<float>(rho), sf, static_cast<float>(rb), scorr);
    b0x = b1x = hx;
    b0y = b1y = hy;
    b0z = b1z = hz;
  } else {
    hi = make_float4(1.0e6f + 16.0f * lane, 1.0e6f, 1.0e6f, 0.f);
    lo = make_float4(0.f, 0.f, 0.f, 0.f);
    gp = make_float4(1.f, 0.f, 1.f, 0.f);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    b0x = fminf(b0x, __shfl_xor_sync(kAll, b0x, o));
    b0y = fminf(b0y, __shfl_xor_sync(kAll, b0y, o));
    b0z = fminf(b0z, __shfl_xor_sync(kAll, b0z, o));
    b1x = fmaxf(b1x, __shfl_xor_sync(kAll, b1x, o));
    b1y = fmaxf(b1y, __shfl_xor_sync(kAll, b1y, o));
    b1z = fmaxf(b1z, __shfl_xor_sync(kAll, b1z, o));
  }
  region<float4>(a, kOffHi)[slot] = hi;
  region<float4>(a, kOffLo)[slot] = lo;
  region<float4>(a, kOffGb)[slot] = gp;
  region<long long>(a, kOffSum)[slot] = 0;
  if (lane == 0) {
    float4 *box = region<float4>(a, kOffBox);
    box[2 * (slot >> 5)] = make_float4(b0x, b0y, b0z, 0.f);
    box[2 * (slot >> 5) + 1] = make_float4(b1x, b1y, b1z, 0.f);
  }
}

// One warp per ordered tile pair (I, J): lane l descreens i-atom I*32+l by
// the 32 j-atoms of tile J (read by broadcast from shared memory) and adds
// its FP32 partial, in fixed point, to the atom's sum.
__global__ void __launch_bounds__(256) k_static_born(const StaticArgs a) {
  __shared__ float4 s_hi[8][32], s_lo[8][32], s_gb[8][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const float4 *hi = region<float4>(a, kOffHi), *lo = region<float4>(a, kOffLo), *gb = region<float4>(a, kOffGb);
  const float4 *box = region<float4>(a, kOffBox);
  long long *sum = region<long long>(a, kOffSum);
  const float cut2 = a.born.cutoff2 * 1.0001f + 1e-3f;
  const long long npairs = static_cast<long long>(a.ntile) * a.ntile;
  const long long nwarps = static_cast<long long>(gridDim.x) * (blockDim.x >> 5);
  for (long long p = static_cast<long long>(blockIdx.x) * (blockDim.x >> 5) + w; p < npairs; p += nwarps) {
    const int I = static_cast<int>(p / a.ntile), J = static_cast<int>(p % a.ntile);
    const float4 al = box[2 * I], ah = box[2 * I + 1], bl = box[2 * J], bh = box[2 * J + 1];
    const float gx = fmaxf(0.0f, fmaxf(al.x - bh.x, bl.x - ah.x));
    const float gy = fmaxf(0.0f, fmaxf(al.y - bh.y, bl.y - ah.y));
    const float gz = fmaxf(0.0f, fmaxf(al.z - bh.z, bl.z - ah.z));
    if (gx * gx + gy * gy + gz * gz > cut2) continue;  // warp-uniform
    const int si = I * 32 + lane, sj = J * 32 + lane;
    const float4 h = hi[si], l = lo[si], g = gb[si];
    s_hi[w][lane] = hi[sj];
    s_lo[w][lane] = lo[sj];
    s_gb[w][lane] = gb[sj];
    __syncwarp();
    const bool vi = si < a.natom;
    float acc = 0.0f;
    for (int j = 0; j < 32; j++) {
      const float4 hj = s_hi[w][j], lj = s_lo[w][j], gj = s_gb[w][j];
      const float dx = (h.x - hj.x) + (l.x - lj.x);
      const float dy = (h.y - hj.y) + (l.y - lj.y);
      const float dz = (h.z - hj.z) + (l.z - lj.z);
      const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      const bool in = vi && (J * 32 + j) < a.natom && (J * 32 + j) != si && r2 <= a.born.cutoff2;
      if (in) {
        const float d1 = rsqrt_nr(r2);
        const float t = descreen(a.born, r2 * d1, r2, d1, g.x, gj.y);
        acc += fmaf(t, gj.w, t);
      }
    }
    if (vi && acc != 0.0f)
      atomicAdd(reinterpret_cast<unsigned long long *>(&sum[si]),
                static_cast<unsigned long long>(__float2ll_rn(acc * static_cast<float>(kSumScale))));
    __syncwarp();
  }
}

// HCT (gb=1) or OBC (gb=2, 5) effective radius of each atom
// (src/sff/eff.c:1711-1733), in FP64.
__global__ void k_static_finish(const StaticArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.natom) return;
  const double rb = region<double>(a, kOffRb)[i], ri = rb - a.offset;
  const double sumi = -static_cast<double>(region<long long>(a, kOffSum)[i]) * (1.0 / kSumScale);
  double reff;
  if (a.gb == 1) {
    reff = 1.0 / (1.0 / ri + sumi);
    if (reff < 0.0) reff = 30.0;
  } else {
    const double al = a.gb == 2 ? 0.8 : 1.0, be = a.gb == 2 ? 0.0 : 0.8, ga = a.gb == 2 ? 2.909125 : 4.85;
    const double psi = -ri * sumi;
    const double th = tanh((al - be * psi + ga * psi * psi) * psi);
    reff = 1.0 / (1.0 / ri - th / rb);
  }
  region<double>(a, kOffReff)[i] = reff;
}

// The device address of g_scratch in the current device's context.  Host
// code must not use the symbol itself: in host code it names a host-side
// stand-in, not device memory.
int scratch_for_current_device(unsigned char **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return SFFG_ENODEV;
  void *p = nullptr;
  if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return SFFG_ECUDA;
  *out = static_cast<unsigned char *>(p);
  return SFFG_OK;
}

// A failure after work was queued: wait for that work (it may still read the
// caller's host arrays or write reff) before reporting the error.
int fail_after_queue(cudaStream_t st) {
  cudaStreamSynchronize(st);
  return SFFG_ECUDA;
}

}  // namespace
}  // namespace sffg

extern "C" int sffg_born_radii_static(int natom, const double *x, const double *rborn, const double *fs, int gb,
                                      double rgbmax, double *reff, void *stream) {
  using namespace sffg;
  if (natom > kStaticMaxAtoms) return SFFG_ENOMEM;  // does not fit the static scratch
  if (natom < 1 || !x || !rborn || !fs || !reff) return SFFG_EINVAL;
  if (!(gb == 1 || gb == 2 || gb == 5) || !(rgbmax > 0.0)) return SFFG_EINVAL;
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : cudaStreamLegacy;
  // copies from pageable host memory and the final wait are illegal on a
  // capturing stream and would invalidate the caller's capture: refuse
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) return SFFG_ECUDA;
  if (cap != cudaStreamCaptureStatusNone) return SFFG_EINVAL;
  // an error left by an earlier, unrelated call would otherwise be reported
  // as this call's launch failure
  (void)cudaGetLastError();
  unsigned char *base = nullptr;
  const int rc = scratch_for_current_device(&base);
  if (rc != SFFG_OK) return rc;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm < 1)
    return SFFG_ECUDA;

  // Largest screened radius: bounds the pair distance that descreens at all.
  double smax = 0.0;
  for (int i = 0; i < natom; i++) {
    const double s = fs[i] * (rborn[i] - 0.09);
    if (s > smax) smax = s;
  }
  StaticArgs a;
  a.base = base;
  a.natom = natom;
  a.ntile = (natom + 31) / 32;
  a.gb = gb;
  a.offset = 0.09;  // src/sff/sff.c:1330 (gb 1, 2 and 5)
  a.born.rgbmax = static_cast<float>(rgbmax);
  a.born.rgbmax1i = static_cast<float>(1.0 / rgbmax);
  a.born.rgbmax2i = static_cast<float>(1.0 / (rgbmax * rgbmax));
  const double c = rgbmax + smax;
  a.born.cutoff2 = static_cast<float>(c * c);

  const size_t n = static_cast<size_t>(natom);
  if (cudaMemcpyAsync(base + kOffX, x, 3 * n * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(base + kOffRb, rborn, n * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(base + kOffFs, fs, n * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return fail_after_queue(st);
  k_static_pack<<<a.ntile, 32, 0, st>>>(a);
  // eight warps per block, eight resident blocks per SM at most
  const long long warps = static_cast<long long>(a.ntile) * a.ntile;
  const long long cap_blocks = 8LL * nsm;
  const int blocks = static_cast<int>(warps / 8 + 1 < cap_blocks ? warps / 8 + 1 : cap_blocks);
  k_static_born<<<blocks, 256, 0, st>>>(a);
  k_static_finish<<<(natom + 127) / 128, 128, 0, st>>>(a);
  if (cudaGetLastError() != cudaSuccess) return fail_after_queue(st);
  if (cudaMemcpyAsync(reff, base + kOffReff, n * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return fail_after_queue(st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return SFFG_ECUDA;
  return SFFG_OK;
}
