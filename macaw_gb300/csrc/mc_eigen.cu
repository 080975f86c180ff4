// mc_eigen.cu -- k-eigenvalue bank processing between generations: the
// fixed-order sums of the keff estimators, the fission bank's sort into
// (parent id, progeny index) order and its resampling into the next
// generation's source sites.
//
// The steps restate, for one GPU, what OpenMC's finalize_generation does
// for OpenMCStudy::postExecuteStudy on one rank
// (src/userobjects/OpenMCStudy.C:374-402): sort_fission_bank, then
// synchronize_bank -- the algorithm OpenMCStudy::synchronizeBanks adapts
// (src/userobjects/OpenMCStudy.C:430-607) -- with each site's draw taken by
// skip-ahead from the generation's tracking-stream seed instead of one
// sequential loop, and every prefix sum done by scans.  All of it is
// integer and copy work bound by HBM bandwidth; none of it is on the
// per-segment path.
#include "mc_kernels.h"

namespace mc {

namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanPer = 8;
constexpr int64_t kScanTile = (int64_t)kScanThreads * kScanPer;

__global__ void __launch_bounds__(kReduceTile) k_tile_sums(const double* __restrict__ v, int64_t n,
                                                           double* __restrict__ part) {
  __shared__ double t[kReduceTile];
  const int64_t i = (int64_t)blockIdx.x * kReduceTile + threadIdx.x;
  t[threadIdx.x] = i < n ? v[i] : 0.0;
  __syncthreads();
  for (int s = kReduceTile / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) t[threadIdx.x] = t[threadIdx.x] + t[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = t[0];
}

// Exclusive scan over the 1024 per-thread values of a block (in place in
// sh); returns the block total.
__device__ __forceinline__ int64_t block_exclusive_scan(int64_t* sh, int64_t mine) {
  const int t = threadIdx.x;
  sh[t] = mine;
  __syncthreads();
  for (int o = 1; o < kScanThreads; o <<= 1) {
    const int64_t v = t >= o ? sh[t - o] : 0;
    __syncthreads();
    sh[t] += v;
    __syncthreads();
  }
  const int64_t total = sh[kScanThreads - 1];
  const int64_t excl = sh[t] - mine;
  __syncthreads();
  sh[t] = excl;
  __syncthreads();
  return total;
}

// Per tile of kScanTile counts: its sum.
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const int* __restrict__ cnt, int64_t n,
                                                             int64_t* __restrict__ tile) {
  __shared__ int64_t sh[kScanThreads];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPer;
  int64_t mine = 0;
  for (int k = 0; k < kScanPer; ++k)
    if (base + k < n) mine += cnt[base + k];
  const int64_t total = block_exclusive_scan(sh, mine);
  if (threadIdx.x == 0) tile[blockIdx.x] = total;
}

// Exclusive scan of the nt tile sums in one block; off_n receives the total.
__global__ void __launch_bounds__(kScanThreads) k_scan_top(int64_t* __restrict__ tile, int64_t nt,
                                                           int64_t* __restrict__ off_n) {
  __shared__ int64_t sh[kScanThreads];
  const int64_t per = (nt + kScanThreads - 1) / kScanThreads;
  const int64_t b0 = (int64_t)threadIdx.x * per;
  int64_t mine = 0;
  for (int64_t i = b0; i < b0 + per && i < nt; ++i) mine += tile[i];
  const int64_t total = block_exclusive_scan(sh, mine);
  int64_t run = sh[threadIdx.x];
  for (int64_t i = b0; i < b0 + per && i < nt; ++i) {
    const int64_t c = tile[i];
    tile[i] = run;
    run += c;
  }
  if (threadIdx.x == 0) *off_n = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const int* __restrict__ cnt, int64_t n,
                                                             const int64_t* __restrict__ tile,
                                                             int64_t* __restrict__ off) {
  __shared__ int64_t sh[kScanThreads];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPer;
  int c[kScanPer];
  int64_t mine = 0;
  for (int k = 0; k < kScanPer; ++k) {
    c[k] = base + k < n ? cnt[base + k] : 0;
    mine += c[k];
  }
  block_exclusive_scan(sh, mine);
  int64_t run = tile[blockIdx.x] + sh[threadIdx.x];
  for (int k = 0; k < kScanPer; ++k) {
    if (base + k < n) off[base + k] = run;
    run += c[k];
  }
}

// Sites banked beyond a history's recorded count, or by a history outside
// the generation, cannot occur (sites are counted where they are made); the
// guard keeps a corrupt bank from writing out of bounds.
__global__ void k_bank_sort(const mc_fission_site* __restrict__ in, int64_t m, const int64_t* __restrict__ off,
                            int64_t first, int64_t n_hist, mc_fission_site* __restrict__ out) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
    const mc_fission_site o = in[i];
    const int64_t h = o.parent - 1 - first;
    if (h < 0 || h >= n_hist) continue;
    const int64_t pos = off[h] + o.progeny;
    if (o.progeny < 0 || pos >= off[h + 1] || pos >= m) continue;
    out[pos] = o;
  }
}

// OpenMC synchronize_bank: the i-th sorted site is copied `copies` times
// (n_particles / total when fewer sites than particles were banked) and
// once more when the i-th draw of the generation's stream is below p.
__global__ void k_bank_counts(int64_t m, uint64_t seed0, int copies, double p, int* __restrict__ cnt) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
    const Skip k = skip_ahead((uint64_t)i);
    uint64_t s = k.G * seed0 + k.C;
    const double xi = prn(s);
    cnt[i] = copies + (xi < p ? 1 : 0);
  }
}

__device__ __forceinline__ mc_site as_site(const mc_fission_site& f) {
  mc_site o;
  o.x = f.x;
  o.y = f.y;
  o.z = f.z;
  o.u = f.u;
  o.v = f.v;
  o.w = f.w;
  o.E = f.E;
  o.wgt = f.wgt;
  return o;
}

// Copies of site i fill [pos[i], pos[i+1]) up to n (a too long resampled
// bank is cut at n particles).
__global__ void k_bank_fill(const mc_fission_site* __restrict__ sorted, int64_t m, const int64_t* __restrict__ pos,
                            int64_t n, mc_site* __restrict__ src) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
    const int64_t a = pos[i];
    if (a >= n) continue;
    const int64_t b = pos[i + 1] < n ? pos[i + 1] : n;
    if (b <= a) continue;
    const mc_site o = as_site(sorted[i]);
    for (int64_t j = a; j < b; ++j) src[j] = o;
  }
}

// A too short resampled bank is completed with the last sites of the
// sorted bank: entry finish + j takes site max(0, m - need + j).
__global__ void k_bank_pad(const mc_fission_site* __restrict__ sorted, int64_t m, const int64_t* __restrict__ pos,
                           int64_t n, mc_site* __restrict__ src) {
  const int64_t fin = pos[m];
  if (fin >= n) return;
  const int64_t need = n - fin;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < need; j += stride) {
    int64_t k = m - need + j;
    if (k < 0) k = 0;
    src[fin + j] = as_site(sorted[k]);
  }
}

int grid_for(int64_t n) {
  const int64_t g = (n + 255) / 256;
  return (int)(g < 1 ? 1 : (g > 4864 ? 4864 : g));
}

}  // namespace

cudaError_t launch_tile_sums(const double* v, int64_t n, double* part, cudaStream_t st) {
  const int64_t nt = (n + kReduceTile - 1) / kReduceTile;
  if (nt > 0) k_tile_sums<<<(unsigned)nt, kReduceTile, 0, st>>>(v, n, part);
  return cudaGetLastError();
}

int64_t scan_tmp_size(int64_t n) { return (n + kScanTile - 1) / kScanTile + 1; }

cudaError_t launch_scan(const int* cnt, int64_t n, int64_t* off, int64_t* tmp, cudaStream_t st) {
  const int64_t nt = (n + kScanTile - 1) / kScanTile;
  if (nt == 0) return cudaMemsetAsync(off, 0, sizeof(int64_t), st);
  k_scan_tiles<<<(unsigned)nt, kScanThreads, 0, st>>>(cnt, n, tmp);
  k_scan_top<<<1, kScanThreads, 0, st>>>(tmp, nt, off + n);
  k_scan_apply<<<(unsigned)nt, kScanThreads, 0, st>>>(cnt, n, tmp, off);
  return cudaGetLastError();
}

cudaError_t launch_bank_sort(const mc_fission_site* in, int64_t m, const int64_t* off, int64_t first, int64_t n_hist,
                             mc_fission_site* out, cudaStream_t st) {
  if (m > 0) k_bank_sort<<<grid_for(m), 256, 0, st>>>(in, m, off, first, n_hist, out);
  return cudaGetLastError();
}

cudaError_t launch_bank_counts(int64_t m, uint64_t seed0, int copies, double p, int* cnt, cudaStream_t st) {
  if (m > 0) k_bank_counts<<<grid_for(m), 256, 0, st>>>(m, seed0, copies, p, cnt);
  return cudaGetLastError();
}

cudaError_t launch_bank_fill(const mc_fission_site* sorted, int64_t m, const int64_t* pos, int64_t n, mc_site* src,
                             cudaStream_t st) {
  if (m > 0) {
    k_bank_fill<<<grid_for(m), 256, 0, st>>>(sorted, m, pos, n, src);
    k_bank_pad<<<grid_for(n), 256, 0, st>>>(sorted, m, pos, n, src);
  }
  return cudaGetLastError();
}

}  // namespace mc
