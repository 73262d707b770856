// gf_sino.cu -- sinogram-domain kernels: the subset-local (radial-major,
// padded-row) layouts the projectors use, the data/projection ratio, the
// normalization mask and the VLOR count/split.
//
// Elements of a subset-layout array are indexed by
//   (angle-in-subset tl, radial bin r, padded row p): (tl*NRAD + r)*PS + p,
// with one array holding every subset back to back when it is static.
#include <cub/device/device_radix_sort.cuh>

#include "gf_kernels.h"

namespace gf {

__device__ __forceinline__ size_t file_lor(const DevGeom& g, int seg, int plane, int theta, int r) {
  const DevSeg& sg = g.seg[seg];
  return ((size_t)(plane - sg.zmin) + sg.acc) * ((size_t)g.nrad * g.nang) + (size_t)theta * g.nrad + r;
}

// rowmap entries: (seg, plane) for real rows; (seg, -1 - edge) for pad rows,
// edge 0 = before the block, 1 = after; (-1, -1) past PP.
__device__ __forceinline__ bool resolve_row(const DevGeom& g, int2 m, int* seg, int* plane) {
  if (m.x < 0) return false;
  *seg = m.x;
  if (m.y >= 0) {
    *plane = m.y;
    return true;
  }
  if (m.x != 0) return false;  // oblique pad row: sentinel
  *plane = (m.y == -1) ? 0 : g.nzs - 1;
  return true;
}

// Rank of angle theta in the all-subset layout: subsets are stored in order,
// subset s = theta % nsub holding angles s, s + nsub, ...; the first
// nang % nsub subsets hold one angle more than the others.
__device__ __forceinline__ int angle_rank(const DevGeom& g, int theta) {
  const int s = theta % g.nsub, l = theta / g.nsub;
  const int q = g.nang / g.nsub, rem = g.nang % g.nsub;
  return s * q + min(s, rem) + l;
}

// The static subset layouts are a transpose of the file layout: for one
// angle, file element (plane, radial) goes to (radial, padded row).  A block
// moves a tile of 32 radial bins x 32 padded rows through shared memory, so
// both the file reads (along radial bins) and the layout writes (along rows)
// are whole 128-byte lines.

// (data*RES, max(bg*RES, 0)) for every subset, from the parsed file
// (2*NDATA floats: prompts then background).  GFIRST.cu:224-226, 423.
// Pad rows hold (0, 0).
__global__ void __launch_bounds__(256) build_dbg_kernel(const DevGeom g, const int2* __restrict__ rowmap,
                                                        const float* __restrict__ sino2, float2* __restrict__ dbg,
                                                        size_t ndata) {
  __shared__ float2 tile[32][33];
  const int r0 = blockIdx.x * 32, p0 = blockIdx.y * 32, theta = blockIdx.z;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const float res = (float)g.res;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int p = p0 + ty + 8 * k, r = r0 + tx;
    float2 v = make_float2(0.f, 0.f);
    if (p < g.PS && r < g.nrad) {
      const int2 m = rowmap[p];
      if (m.x >= 0 && m.y >= 0) {
        const size_t lor = file_lor(g, m.x, m.y, theta, r);
        const float bg = __fmul_rn(res, sino2[ndata + lor]);
        v = make_float2(__fmul_rn(res, sino2[lor]), ((double)bg < 0.) ? 0.f : bg);
      }
    }
    tile[ty + 8 * k][tx] = v;
  }
  __syncthreads();
  const size_t base = (size_t)angle_rank(g, theta) * g.nrad;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int r = r0 + ty + 8 * k, p = p0 + tx;
    if (r < g.nrad && p < g.PS) dbg[(base + r) * g.PS + p] = tile[tx][ty + 8 * k];
  }
}

cudaError_t launch_build_dbg(const DevGeom& g, const int2* rowmap, const float* sino2, float2* dbg,
                             cudaStream_t st) {
  const size_t ndata = (size_t)g.P * g.nang * g.nrad;
  const dim3 grid((g.nrad + 31) / 32, (g.PS + 31) / 32, g.nang);
  build_dbg_kernel<<<grid, dim3(32, 8), 0, st>>>(g, rowmap, sino2, dbg, ndata);
  return cudaGetLastError();
}

// Normalization mask per subset element, GFIRST.cu:447, 453-458: 1 where
// proj_blank > 0.01 and blank > 0.01, else -1000; oblique pad rows -1000,
// segment 0's pad rows repeat its first/last plane.
__global__ void __launch_bounds__(256) build_cal_kernel(const DevGeom g, const int2* __restrict__ rowmap,
                                                        const float* __restrict__ proj_ref,
                                                        const float* __restrict__ norm, float* __restrict__ cal) {
  __shared__ float tile[32][33];
  const int r0 = blockIdx.x * 32, p0 = blockIdx.y * 32, theta = blockIdx.z;
  const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int p = p0 + ty + 8 * k, r = r0 + tx;
    float v = -1000.f;
    int seg, plane;
    if (p < g.PS && r < g.nrad && resolve_row(g, rowmap[p], &seg, &plane)) {
      const size_t lor = file_lor(g, seg, plane, theta, r);
      v = ((double)proj_ref[lor] > 0.01 && (double)norm[lor] > 0.01) ? 1.0f : -1000.f;
    }
    tile[ty + 8 * k][tx] = v;
  }
  __syncthreads();
  const size_t base = (size_t)angle_rank(g, theta) * g.nrad;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int r = r0 + ty + 8 * k, p = p0 + tx;
    if (r < g.nrad && p < g.PS) cal[(base + r) * g.PS + p] = tile[tx][ty + 8 * k];
  }
}

cudaError_t launch_build_cal(const DevGeom& g, const int2* rowmap, const float* proj_ref, const float* norm,
                             float* cal, cudaStream_t st) {
  const dim3 grid((g.nrad + 31) / 32, (g.PS + 31) / 32, g.nang);
  build_cal_kernel<<<grid, dim3(32, 8), 0, st>>>(g, rowmap, proj_ref, norm, cal);
  return cudaGetLastError();
}

__device__ __forceinline__ float ratio_rule(float proj, float data, float bg) {
  // GFIRST.cu:423-429
  if ((double)bg < 0.) bg = 0.f;
  const float s = __fadd_rn(proj, bg);
  return (s >= 0.01f) ? __fdiv_rn(data, s) : -1000.f;
}

// (corr, calib) pairs of one subset from file-layout corr and calib.
__global__ void corrcal_from_file_kernel(const DevGeom g, const int2* __restrict__ rowmap, int subset,
                                         const float* __restrict__ corr, const float* __restrict__ calib,
                                         float2* __restrict__ cc, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int p = (int)(i % g.PS);
  const size_t q = i / g.PS;
  const int r = (int)(q % g.nrad), tl = (int)(q / g.nrad);
  const int theta = subset_angle(g, subset, tl);
  int seg, plane;
  float2 v = make_float2(-1000.f, -1000.f);
  if (resolve_row(g, rowmap[p], &seg, &plane)) {
    const size_t lor = file_lor(g, seg, plane, theta, r);
    v = make_float2(corr[lor], calib[lor]);
  }
  cc[i] = v;
}

cudaError_t launch_corrcal_from_file(const DevGeom& g, const int2* rowmap, int subset, int na, const float* corr,
                                     const float* calib, float2* corrcal, cudaStream_t st) {
  const size_t n = (size_t)na * g.nrad * g.PS;
  corrcal_from_file_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(g, rowmap, subset, corr, calib, corrcal, n);
  return cudaGetLastError();
}

// Ratio for the VLOR triples (GFIRST.cu:415-430 with val_dato = datos_v*RES,
// GFIRST.cu:397, 421) written as (corr, calib) pairs of one subset.
template <class Pair>
__global__ void ratio_gather_kernel(const DevGeom g, const int2* __restrict__ rowmap, int subset,
                                    const float* __restrict__ proj_full, const float* __restrict__ datos_v,
                                    const float2* __restrict__ dbg_t, const float* __restrict__ cal,
                                    Pair* __restrict__ cc, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int p = (int)(i % g.PS);
  const size_t q = i / g.PS;
  const int r = (int)(q % g.nrad), tl = (int)(q / g.nrad);
  const int theta = subset_angle(g, subset, tl);
  int seg, plane;
  float2 v = make_float2(-1000.f, -1000.f);
  const int2 m = rowmap[p];
  if (resolve_row(g, m, &seg, &plane)) {
    const size_t lor = file_lor(g, seg, plane, theta, r);
    // the edge row's own element for segment 0's pad rows
    const int prow = (m.y >= 0) ? p : (m.y == -1 ? p + 1 : p - 1);
    const size_t e = i - p + prow;
    const float data = __fmul_rn(datos_v[lor], (float)g.res);
    v = make_float2(ratio_rule(proj_full[lor], data, dbg_t[e].y), cal[e]);
  }
  cc[i] = pair_from<Pair>(v);
}

cudaError_t launch_ratio_gather(const DevGeom& g, const int2* rowmap, int subset, int na, const float* proj_full,
                                const float* datos_v, const float2* dbg_t, const float* cal, void* corrcal,
                                int storage, cudaStream_t st) {
  const size_t n = (size_t)na * g.nrad * g.PS;
  const unsigned nb = (unsigned)((n + 255) / 256);
  switch (storage) {
    case 0: ratio_gather_kernel<<<nb, 256, 0, st>>>(g, rowmap, subset, proj_full, datos_v, dbg_t, cal, static_cast<float2*>(corrcal), n); break;
    case 1: ratio_gather_kernel<<<nb, 256, 0, st>>>(g, rowmap, subset, proj_full, datos_v, dbg_t, cal, static_cast<__half2*>(corrcal), n); break;
    case 2: ratio_gather_kernel<<<nb, 256, 0, st>>>(g, rowmap, subset, proj_full, datos_v, dbg_t, cal, static_cast<__nv_bfloat162*>(corrcal), n); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// File-layout ratio over one subset's bins (operator entry point).
__global__ void ratio_file_kernel(const DevGeom g, int subset, const float* __restrict__ proj,
                                  const float* __restrict__ data, const float* __restrict__ bg,
                                  float* __restrict__ corr, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int theta = (int)((i / g.nrad) % g.nang);
  if (theta % g.nsub != subset) return;
  corr[i] = ratio_rule(proj[i], data[i], bg[i]);
}

cudaError_t launch_ratio_file(const DevGeom& g, int subset, const float* proj, const float* data, const float* bg,
                              float* corr, cudaStream_t st) {
  const size_t n = (size_t)g.P * g.nang * g.nrad;
  ratio_file_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(g, subset, proj, data, bg, corr, n);
  return cudaGetLastError();
}

__global__ void norm_mask_kernel(const float* __restrict__ pb, const float* __restrict__ b, float* __restrict__ c,
                                 size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  c[i] = ((double)pb[i] > 0.01 && (double)b[i] > 0.01) ? 1.0f : -1000.f;
}

// *flag = 1 when a and b differ anywhere in their n floats (bitwise); *flag
// must hold 0 before.
__global__ void differs_kernel(const float* __restrict__ a, const float* __restrict__ b, size_t n, int* flag) {
  int d = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    d |= __float_as_int(a[i]) ^ __float_as_int(b[i]);
  if (__any_sync(0xffffffffu, d != 0) && (threadIdx.x & 31) == 0) atomicExch(flag, 1);
}

cudaError_t launch_differs(const float* a, const float* b, size_t n, int* flag, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  differs_kernel<<<1216, 256, 0, st>>>(a, b, n, flag);
  return cudaGetLastError();
}

cudaError_t launch_norm_mask(const DevGeom& g, const float* proj_blank, const float* blank, float* calib,
                             cudaStream_t st) {
  const size_t n = (size_t)g.P * g.nang * g.nrad;
  norm_mask_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(proj_blank, blank, calib, n);
  return cudaGetLastError();
}

// ---- VLOR, GFIRST.cu:229-247, 373-389 --------------------------------------
__device__ __forceinline__ bool vlor_bins(const int32_t* ev, long long e, long long ndata, long long* i1,
                                          long long* i2) {
  *i1 = (long long)ev[2 * e] - 1;
  *i2 = (long long)ev[2 * e + 1] - 1;
  return !(*i1 <= 0 || *i2 <= 0 || *i1 >= ndata || *i2 >= ndata);
}

__global__ void vlor_count_kernel(const int32_t* __restrict__ ev, long long nev, long long ndata, float* cnt) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nev) return;
  long long i1, i2;
  if (!vlor_bins(ev, e, ndata, &i1, &i2)) return;
  atomicAdd(cnt + i1, 1.0f);
  atomicAdd(cnt + i2, 1.0f);
}

cudaError_t launch_vlor_count(const DevGeom& g, const int32_t* ev, long long nev, float* cnt, cudaStream_t st) {
  if (nev <= 0) return cudaSuccess;
  const long long ndata = (long long)g.P * g.nang * g.nrad;
  vlor_count_kernel<<<(unsigned)((nev + 255) / 256), 256, 0, st>>>(ev, nev, ndata, cnt);
  return cudaGetLastError();
}

// BLANKT[i] = datos_t[i]/float(RES*cnt) where cnt > 0.01 (datos_t = RES*file).
__global__ void blankt_kernel(const float* __restrict__ cnt, const float* __restrict__ t, float res, float* bl,
                              size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float val = cnt[i];
  bl[i] = ((double)val > 0.01) ? __fdiv_rn(__fmul_rn(res, t[i]), __fmul_rn(res, val)) : 0.f;
}

cudaError_t launch_blankt(const DevGeom& g, const float* cnt, const float* tsino_raw, float* blankt,
                          cudaStream_t st) {
  const size_t n = (size_t)g.P * g.nang * g.nrad;
  blankt_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(cnt, tsino_raw, (float)g.res, blankt, n);
  return cudaGetLastError();
}

// ---- VLOR split in the reference's order ------------------------------------
// The reference adds each event's two shares to their bins in file order
// (GFIRST.cu:373-389), so a bin's sum is its shares added in event order.
// One 64-bit key per event end, (bin << 32) | (2*event + end), sorted once,
// puts each bin's shares in that order; the split then sums each bin's run
// sequentially: the same additions in the same order, without atomics.
constexpr unsigned long long kNoKey = ~0ull;  // an end of a rejected event

__global__ void vlor_keys_kernel(const int32_t* __restrict__ ev, long long nev, long long ndata,
                                 unsigned long long* keys) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nev) return;
  long long i1, i2;
  const bool ok = vlor_bins(ev, e, ndata, &i1, &i2);
  keys[2 * e] = ok ? ((unsigned long long)i1 << 32) | (unsigned long long)(2 * e) : kNoKey;
  keys[2 * e + 1] = ok ? ((unsigned long long)i2 << 32) | (unsigned long long)(2 * e + 1) : kNoKey;
}

size_t vlor_sort_temp_bytes(long long nev) {
  size_t bytes = 0;
  cub::DeviceRadixSort::SortKeys(nullptr, bytes, (const unsigned long long*)nullptr,
                                 (unsigned long long*)nullptr, (int)(2 * nev), 0, 64);
  return bytes;
}

cudaError_t launch_vlor_sort(const DevGeom& g, const int32_t* ev, long long nev, unsigned long long* keys_tmp,
                             unsigned long long* keys, void* temp, size_t temp_bytes, cudaStream_t st) {
  if (nev <= 0) return cudaSuccess;
  if (nev >= (1ll << 30)) return cudaErrorInvalidValue;  // 2*event + end must fit 32 bits, counts an int
  const long long ndata = (long long)g.P * g.nang * g.nrad;
  vlor_keys_kernel<<<(unsigned)((nev + 255) / 256), 256, 0, st>>>(ev, nev, ndata, keys_tmp);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return cub::DeviceRadixSort::SortKeys(temp, temp_bytes, keys_tmp, keys, (int)(2 * nev), 0, 64, st);
}

// pass 1, over events: both shares of each event, share[2e + end]
__global__ void vlor_shares_kernel(const int32_t* __restrict__ ev, long long nev, long long ndata,
                                   const float* __restrict__ proj, const float* __restrict__ bl, float* share) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nev) return;
  long long i1, i2;
  if (!vlor_bins(ev, e, ndata, &i1, &i2)) return;  // its keys are kNoKey: never read
  const float valor = __fadd_rn(bl[i1], bl[i2]);
  const float s1 = proj[i1], s2 = proj[i2];
  const float s = __fadd_rn(s1, s2);
  const float s_inv = (s > 0.01f) ? (float)__drcp_rn((double)s) : 0.f;
  share[2 * e] = __fmul_rn(__fmul_rn(s1, s_inv), valor);
  share[2 * e + 1] = __fmul_rn(__fmul_rn(s2, s_inv), valor);
}

// pass 2, over the sorted ends: the first end of each bin adds the bin's
// shares in event order
__global__ void vlor_split_sorted_kernel(const unsigned long long* __restrict__ keys, long long n,
                                         const float* __restrict__ share, float* out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned long long k = keys[i];
  if (k == kNoKey) return;
  const unsigned long long bin = k >> 32;
  if (i > 0 && (keys[i - 1] >> 32) == bin) return;  // not the first share of its bin
  float sum = out[bin];  // the shares are added to out, as the reference adds them to SINOG_VLOR
  for (long long j = i; j < n && (keys[j] >> 32) == bin; j++) sum = __fadd_rn(sum, share[keys[j] & 0xffffffffull]);
  out[bin] = sum;
}

cudaError_t launch_vlor_split_sorted(const DevGeom& g, const unsigned long long* keys, long long nev,
                                     const int32_t* ev, const float* proj, const float* blankt, float* share,
                                     float* out, cudaStream_t st) {
  if (nev <= 0) return cudaSuccess;
  const long long ndata = (long long)g.P * g.nang * g.nrad;
  vlor_shares_kernel<<<(unsigned)((nev + 255) / 256), 256, 0, st>>>(ev, nev, ndata, proj, blankt, share);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const long long n = 2 * nev;
  vlor_split_sorted_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(keys, n, share, out);
  return cudaGetLastError();
}

// ---- VLOR events given as LOR endpoints -----------------------------------
// One LOR (x1,y1,z1,x2,y2,z2 in mm; x/y about the axis, z about the axial
// centre) -> 0-based sinogram bin, or -1.  Inverse of gf_bin_endpoints.
__device__ long long lor_bin(const DevGeom& g, const float* e, float vx, float hs, float pi_ref) {
  const float dx = e[3] - e[0], dy = e[4] - e[1], dzm = e[5] - e[2];
  const float L = sqrtf(dx * dx + dy * dy);
  if (!(L > 0.f)) return -1;
  float ux = dx / L, uy = dy / L, sgn = 1.f;
  // direction (sin t, -cos t) with t in (0, pi]
  float th = atan2f(ux, -uy);
  if (th <= 0.f) {
    th += pi_ref;
    sgn = -sgn;
  }
  int t = __float2int_rn((pi_ref - th) * (float)g.nang / pi_ref);
  if (t >= g.nang) {
    t -= g.nang;
    sgn = -sgn;
  }
  if (t < 0) t += g.nang;
  const float2 sc = g.trig[t];  // (sin, cos)
  ux = sgn * (dx / L);
  uy = sgn * (dy / L);
  const float x0mm = e[0] * sc.y + e[1] * sc.x;
  const int ird = __float2int_rn(x0mm / (vx * g.fx_fp) + g.radm);
  if (ird < 0 || ird >= g.nrad) return -1;
  const float slope = sgn * dzm / L * vx / hs;  // slices per voxel step along the ray
  int best = -1;
  float bd = 3.0e38f;
  for (int s = 0; s < g.nseg; s++) {
    const float d = fabsf(g.seg[s].dz - slope);
    if (d < bd) {
      bd = d;
      best = s;
    }
  }
  const DevSeg sg = g.seg[best];
  const float cx = x0mm * sc.y, cy = x0mm * sc.x;
  const float lam1 = ((e[0] - cx) * ux + (e[1] - cy) * uy) / vx;
  const float z0 = e[2] / hs + 0.5f * (float)g.nzs - lam1 * sg.dz;  // texel z at the closest point
  const int iz0 = __float2int_rn(z0 - 0.5f);
  if (iz0 < sg.zmin || iz0 >= g.nzs - sg.zmin) return -1;
  return ((long long)(iz0 - sg.zmin) + sg.acc) * ((long long)g.nrad * g.nang) + (long long)t * g.nrad + ird;
}

__global__ void vlor_endpoints_kernel(const DevGeom g, const float* __restrict__ lors, long long n, float vx, float hs,
                                      float pi_ref, int32_t* __restrict__ ev) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int k = 0; k < 2; k++) {
    const long long b = lor_bin(g, lors + 12 * i + 6 * k, vx, hs, pi_ref);
    ev[2 * i + k] = (int32_t)(b + 1);  // 1-based; 0 = rejected, as the reference rejects i <= 0
  }
}

cudaError_t launch_vlor_endpoints(const DevGeom& g, const float* lors, long long n, float vx, float hs, int32_t* ev,
                                  cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  vlor_endpoints_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(g, lors, n, vx, hs, 3.1415926f, ev);
  return cudaGetLastError();
}

}  // namespace gf
