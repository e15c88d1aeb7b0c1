// Device radix sort and scan shared by the set-up units (sgh_topo.cu,
// sgh_setup.cu); included inside each unit's anonymous namespace.
//   radix_sort: stable LSD sort of (uint64 key, int value) pairs, 8-bit digits,
//               2048 items per block, items ranked in tile order within their
//               digit (warp match + per-warp digit counts), so equal keys keep
//               their input order;
//   exclusive_scan: unsigned counts, per-chunk scan + one-block scan of the
//               chunk totals (up to 8192^2 values).
#pragma once

constexpr int kSortBlock = 256;
constexpr int kTile = 2048;  // radix-sort items per block (8 per thread)

__global__ void __launch_bounds__(kSortBlock) k_hist(int n, const uint64_t* __restrict__ key, int shift,
                                                 unsigned* __restrict__ counts, int nblocks) {
  __shared__ unsigned h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * kTile;
  for (int r = 0; r < kTile / kSortBlock; ++r) {
    const long long i = base + (long long)r * kSortBlock + threadIdx.x;
    if (i < n) atomicAdd(&h[(key[i] >> shift) & 255], 1u);
  }
  __syncthreads();
  counts[(size_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter: items of a tile are ranked in tile order within their digit.
__global__ void __launch_bounds__(kSortBlock) k_scatter(int n, const uint64_t* __restrict__ kin,
                                                    const int* __restrict__ vin, uint64_t* __restrict__ kout,
                                                    int* __restrict__ vout, int shift,
                                                    const unsigned* __restrict__ offsets, int nblocks) {
  __shared__ unsigned run[256];
  __shared__ unsigned wcnt[kSortBlock / 32][256];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  run[threadIdx.x] = offsets[(size_t)threadIdx.x * nblocks + blockIdx.x];
  const long long base = (long long)blockIdx.x * kTile;
  const unsigned lt = (1u << lane) - 1u;
  for (int r = 0; r < kTile / kSortBlock; ++r) {
    for (int w = 0; w < kSortBlock / 32; ++w) wcnt[w][threadIdx.x] = 0;
    __syncthreads();
    const long long i = base + (long long)r * kSortBlock + threadIdx.x;
    const bool live = i < n;
    uint64_t k = 0;
    int v = 0;
    int d = 256 + lane;  // distinct dummy digits for dead lanes
    if (live) {
      k = kin[i];
      v = vin[i];
      d = (int)((k >> shift) & 255);
    }
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
    const unsigned rank = __popc(peers & lt);
    if (live && rank == 0) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    {  // per digit: prefix over the warps of this round, then advance the run
      const int dd = threadIdx.x;
      unsigned acc = run[dd];
      for (int w = 0; w < kSortBlock / 32; ++w) {
        const unsigned c = wcnt[w][dd];
        wcnt[w][dd] = acc;
        acc += c;
      }
      run[dd] = acc;
    }
    __syncthreads();
    if (live) {
      const unsigned pos = wcnt[warp][d] + rank;
      kout[pos] = k;
      vout[pos] = v;
    }
    __syncthreads();
  }
}

// Exclusive scan of unsigned counts: per-chunk scan (1024 threads x 8), chunk
// totals scanned by one block, offsets added.
constexpr int kScanThreads = 1024, kScanPer = 8, kScanChunk = kScanThreads * kScanPer;

__device__ unsigned block_exclusive_scan(unsigned v, unsigned* total) {
  __shared__ unsigned ws[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[warp] = x;
  __syncthreads();
  if (warp == 0) {
    unsigned s = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xFFFFFFFFu, s, o);
      if (lane >= o) s += y;
    }
    ws[lane] = s;
  }
  __syncthreads();
  const unsigned before = (warp > 0 ? ws[warp - 1] : 0) + x - v;
  if (total) *total = ws[(blockDim.x >> 5) - 1];
  __syncthreads();
  return before;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_chunks(long long n, const unsigned* __restrict__ in,
                                                              unsigned* __restrict__ out,
                                                              unsigned* __restrict__ sums) {
  const long long base = (long long)blockIdx.x * kScanChunk + (long long)threadIdx.x * kScanPer;
  unsigned v[kScanPer], s = 0;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    v[k] = base + k < n ? in[base + k] : 0;
    s += v[k];
  }
  unsigned tot;
  unsigned off = block_exclusive_scan(s, &tot);
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    if (base + k < n) out[base + k] = off;
    off += v[k];
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_sums(int m, unsigned* sums) {
  // m <= kScanChunk
  const int base = threadIdx.x * kScanPer;
  unsigned v[kScanPer], s = 0;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    v[k] = base + k < m ? sums[base + k] : 0;
    s += v[k];
  }
  unsigned off = block_exclusive_scan(s, nullptr);
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    if (base + k < m) sums[base + k] = off;
    off += v[k];
  }
}

__global__ void k_scan_add(long long n, unsigned* __restrict__ out, const unsigned* __restrict__ sums) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += sums[i / kScanChunk];
}

struct Scratch {
  std::vector<void*> p;
  ~Scratch() {
    for (void* q : p) cudaFree(q);
  }
  template <typename T>
  int alloc(T** out, size_t n) {
    void* q = nullptr;
    const size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
    if (cudaMalloc(&q, bytes) != cudaSuccess)
      return set_error(FIERRO_ENOMEM, "topology: cudaMalloc(%zu bytes) failed", bytes);
    p.push_back(q);
    *out = static_cast<T*>(q);
    return FIERRO_OK;
  }
};

int exclusive_scan(Scratch& sc, const unsigned* in, unsigned* out, long long n, cudaStream_t st) {
  const long long chunks = (n + kScanChunk - 1) / kScanChunk;
  if (chunks > kScanChunk) return set_error(FIERRO_EINVAL, "topology: scan of %lld values too long", n);
  unsigned* sums = nullptr;
  TRY(sc.alloc(&sums, (size_t)chunks));
  k_scan_chunks<<<(unsigned)chunks, kScanThreads, 0, st>>>(n, in, out, sums);
  k_scan_sums<<<1, kScanThreads, 0, st>>>((int)chunks, sums);
  k_scan_add<<<(unsigned)((n + kSortBlock - 1) / kSortBlock), kSortBlock, 0, st>>>(n, out, sums);
  return FIERRO_OK;
}

// Stable sort of (key, value) by the low `bits` bits of key; the result is in
// k[0], v[0] on return (buffers swapped as needed).
int radix_sort(Scratch& sc, uint64_t** k, int** v, uint64_t* kt, int* vt, int n, int bits, cudaStream_t st) {
  const int nb = (int)((n + kTile - 1) / kTile);
  unsigned *counts = nullptr, *offs = nullptr;
  TRY(sc.alloc(&counts, (size_t)256 * nb));
  TRY(sc.alloc(&offs, (size_t)256 * nb));
  uint64_t* ka = *k;
  int* va = *v;
  uint64_t* kb = kt;
  int* vb = vt;
  for (int shift = 0; shift < bits; shift += 8) {
    k_hist<<<nb, kSortBlock, 0, st>>>(n, ka, shift, counts, nb);
    TRY(exclusive_scan(sc, counts, offs, (long long)256 * nb, st));
    k_scatter<<<nb, kSortBlock, 0, st>>>(n, ka, va, kb, vb, shift, offs, nb);
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  *k = ka;
  *v = va;
  return FIERRO_OK;
}

