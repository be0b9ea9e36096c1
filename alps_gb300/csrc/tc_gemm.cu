// tc_gemm.cu -- FP64-accurate dense products on the BF16 tensor cores
// (tcgen05.mma, accumulators in tensor memory).
//
// GB300 issues FP64 at a small fraction of its BF16 tensor rate, so the
// dense FP64 products of the setup path (the omega-independent p_perp
// contraction of each k, and the trailing updates of the thin-plate-spline
// LU) run as integer-exact slice products (the Ozaki, Ogita and Oishi
// splitting, 2012):
//
//   * every row of A and every column of B is scaled by a power of two so
//     that its largest element is below 1 in magnitude;
//   * an element x of such a row is written as S = 7 slices of at most 8
//     bits, x = sum_s a_s 2^(-7-8(s-1)), a_s an integer in [-128, 128]
//     (exactly a bfloat16), leaving at most 2^-56 of the row maximum;
//   * the slice pairs (s, t) with s + t <= 8 (28 pairs) are multiplied on
//     the tensor cores; a product of two slices is at most 2^14 and a sum
//     of K <= 256 of them at most 2^22, so with up to four pairs in one FP32
//     accumulator (levels L = s + t <= 5) the accumulators hold exact
//     integers, and the levels above 5 carry 2^-32 of the weight, where
//     FP32 rounding is below 2^-56;
//   * the epilogue reads the seven level accumulators from tensor memory
//     and sums them in FP64 with their weights 2^(-14-8(L-2)).
//
// The error of an entry is then at most 10 K 2^-56 2^(eA_r + eB_c), the
// fixed-point scale of its row and column.  Where that is not small against
// the entry's own size (rows and columns whose large elements do not meet,
// see tc_product_checked), the caller's FP64 fallback recomputes the entry.
//
// Kernel structure (one CTA per 128 x 64 output tile, 128 threads):
//   thread 0      streams the operand tiles of each K chunk (32 wide) into
//                 one of two shared-memory stages with cp.async.bulk,
//                 completion on an mbarrier;
//   thread 32     issues the 56 tcgen05.mma of a chunk (28 slice pairs x 2
//                 K steps of 16) into the level accumulators, and commits
//                 each stage back to the producer;
//   all 4 warps   read the accumulators (tcgen05.ld, one TMEM lane per
//                 output row) and write the FP64 results.
// Operands are sliced into the tensor cores' canonical K-major layout
// without swizzle by tc_slice, so each stage is two contiguous bulk copies.
// Every wait is bounded; a timeout sets the error word and the CTA drains
// its copies, frees its tensor memory and returns.
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include "alps_internal.cuh"
#include "tc_gemm.cuh"

namespace {

constexpr int TC_S = TC_SLICES;           // slices per operand
constexpr int TC_KC = 32;                 // K elements per stage
constexpr int TC_MT = 128;                // output rows per CTA (TMEM lanes)
constexpr int TC_NT = 64;                 // output columns per CTA
constexpr int TC_LEVELS = TC_S;           // levels L = 2 .. S+1
constexpr int TC_A_TILE = TC_MT * TC_KC * 2;  // bytes of one A slice tile (8 KB)
constexpr int TC_B_TILE = TC_NT * TC_KC * 2;  // bytes of one B slice tile (4 KB)
constexpr int TC_STAGE = TC_S * (TC_A_TILE + TC_B_TILE);
constexpr int TC_TMEM_COLS = 512;         // 7 levels x 64 columns, rounded to a power of two
constexpr long long TC_WAIT_LIMIT = 4000000000LL;  // clock64 cycles (about 2 s)

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.b32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// waits for the phase with the given parity to complete; false on timeout
__device__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbar_test(bar, parity))
    if (clock64() - t0 > TC_WAIT_LIMIT) return false;
  return true;
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// shared-memory matrix descriptor: canonical K-major layout without swizzle;
// lbo = byte stride between core matrices along K, sbo = along M/N
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of the fifth-generation tensor cores
  return d;                // base offset 0, layout type 0 (no swizzle)
}

// instruction descriptor of kind::f16: BF16 A and B (both K-major), FP32 D
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
          dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}

// byte offset of element (r, k) inside a slice tile of R rows x 32 K: core
// matrices of 8 rows x 8 elements (128 B), four along K (LBO 128 B), row
// groups SBO = 512 B apart
__host__ __device__ __forceinline__ uint32_t tile_off(int r, int k) {
  return (uint32_t)((r >> 3) * 512 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// the slice pairs in issue order: level by level, L = 2 .. S+1
struct PairTable {
  int n;
  unsigned char sa[TC_S * TC_S], sb[TC_S * TC_S], lev[TC_S * TC_S], first[TC_S * TC_S];
};
__constant__ PairTable c_pairs;

// Row exponents and slices of one operand role.  Element (r, k) of the
// operand is src[r*rs + k*ks] * 2^kexp[k] (kexp may be null; -kexp[k] with
// neg_k), r < R, k < K; rows are padded to RT-row tiles, K to 32.
// out: tiles [rt][kc][s][RT x 32 bf16], exps[r] = e with max_k |x| < 2^e.
template <int RT>
__global__ void k_tc_slice(const double* __restrict__ src, long rs, long ks, int R, int K,
                           const int* __restrict__ kexp, int neg_k, int nkc, __nv_bfloat16* __restrict__ out,
                           int* __restrict__ exps) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int Rpad = ((R + RT - 1) / RT) * RT;
  if (warp >= Rpad) return;
  const int r = warp;
  auto val = [&](int k) -> double {
    if (r >= R || k >= K) return 0.0;
    double x = src[(long)r * rs + (long)k * ks];
    if (kexp) x = ldexp(x, neg_k ? -kexp[k] : kexp[k]);
    return x;
  };
  double mx = 0.0;
  for (int k = lane; k < K; k += 32) mx = fmax(mx, fabs(val(k)));
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  int e = 0;
  if (mx > 0.0) {
    frexp(mx, &e);  // mx = m 2^e, m in [0.5, 1): every |x| 2^-e < 1
  }
  if (lane == 0) exps[r] = e;
  const int rt = r / RT, rr = r % RT;
  for (int k = lane; k < nkc * TC_KC; k += 32) {
    double v = ldexp(val(k), -e + 7);  // |v| < 128 ... a_1 = rint(v) in [-128, 128]
    const int kc = k / TC_KC, kk = k % TC_KC;
    unsigned char* base = reinterpret_cast<unsigned char*>(out) + ((size_t)(rt * nkc + kc) * TC_S) * (RT * TC_KC * 2);
#pragma unroll
    for (int s = 0; s < TC_S; ++s) {
      const double a = rint(v);
      *reinterpret_cast<__nv_bfloat16*>(base + (size_t)s * (RT * TC_KC * 2) + tile_off(rr, kk)) =
          __double2bfloat16(a);
      v = ldexp(v - a, 8);
    }
  }
}

struct TcArgs {
  const __nv_bfloat16* A;  // slices of A [mt][kc][s][128 x 32]
  const __nv_bfloat16* B;  // slices of B [nt][kc][s][64 x 32]
  const int* eA;           // row exponents
  const int* eB;           // column exponents
  double* C;               // C[r*crs + c*ccs]
  long crs, ccs;
  int M, N, nkc;
  double alpha, beta;
  int* err;                // error word: 1 = a bounded wait ran out
  double* bound;           // optional: fixed-point error scale 2^(eA+eB) per entry, same strides as C
};

__global__ void __launch_bounds__(128, 1) k_tc_gemm(TcArgs a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[2], empty[2], done;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int mt = blockIdx.x, nt = blockIdx.y;
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem) + 1023) & ~(uintptr_t)1023);
  if (tid == 0) {
    mbar_init(&full[0], 1);
    mbar_init(&full[1], 1);
    mbar_init(&empty[0], 1);
    mbar_init(&empty[1], 1);
    mbar_init(&done, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) tmem_alloc(&tmem_base, TC_TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = tmem_base;
  const int nkc = a.nkc;
  const size_t a_chunk = (size_t)TC_S * TC_A_TILE, b_chunk = (size_t)TC_S * TC_B_TILE;
  int issued = 0;  // stages the producer filled (thread 0)
  if (tid == 0) {
    // producer
    for (int kc = 0; kc < nkc; ++kc) {
      const int s = kc & 1;
      if (kc >= 2 && !mbar_wait(&empty[s], ((kc >> 1) - 1) & 1)) {
        atomicExch(&abort_flag, 1);
        break;
      }
      if (*((volatile int*)&abort_flag)) break;
      unsigned char* st = sm + (size_t)s * TC_STAGE;
      mbar_expect_tx(&full[s], (uint32_t)(a_chunk + b_chunk));
      bulk_g2s(st, reinterpret_cast<const unsigned char*>(a.A) + ((size_t)mt * nkc + kc) * a_chunk,
               (uint32_t)a_chunk, &full[s]);
      bulk_g2s(st + a_chunk, reinterpret_cast<const unsigned char*>(a.B) + ((size_t)nt * nkc + kc) * b_chunk,
               (uint32_t)b_chunk, &full[s]);
      issued = kc + 1;
    }
  } else if (tid == 32) {
    // MMA issuer
    const uint32_t idesc = idesc_bf16(TC_MT, TC_NT);
    bool ok = true;
    for (int kc = 0; kc < nkc && ok; ++kc) {
      const int s = kc & 1;
      if (!mbar_wait(&full[s], (kc >> 1) & 1)) {
        atomicExch(&abort_flag, 1);
        ok = false;
        break;
      }
      tc_fence_after();
      const uint32_t st = smem_u32(sm + (size_t)s * TC_STAGE);
      for (int q = 0; q < c_pairs.n; ++q) {
        const int sa = c_pairs.sa[q], sb = c_pairs.sb[q], L = c_pairs.lev[q];
        const uint32_t dcol = tbase + (uint32_t)((L - 2) * TC_NT);
#pragma unroll
        for (int ksub = 0; ksub < 2; ++ksub) {
          const uint64_t ad = smem_desc(st + sa * TC_A_TILE + ksub * 256, 128, 512);
          const uint64_t bd = smem_desc(st + (uint32_t)a_chunk + sb * TC_B_TILE + ksub * 256, 128, 512);
          const uint32_t acc = (kc > 0 || ksub > 0 || !c_pairs.first[q]) ? 1u : 0u;
          mma_bf16(dcol, ad, bd, idesc, acc);
        }
      }
      mma_commit(&empty[s]);
    }
    mma_commit(&done);  // arrives once every MMA issued so far has completed
  }
  __syncwarp();
  // epilogue: the 128 threads read one accumulator lane (output row) each
  const bool waited = mbar_wait(&done, 0);
  tc_fence_after();
  __syncthreads();
  if (tid == 0) {
    // drain: every bulk copy the producer issued has landed before the CTA
    // can release its shared memory (bounded; a stage whose MMAs were
    // consumed has completed already)
    for (int kc = (issued > 2 ? issued - 2 : 0); kc < issued; ++kc) mbar_wait(&full[kc & 1], (kc >> 1) & 1);
  }
  if (!waited || abort_flag) {
    if (tid == 0) atomicExch(a.err, 1);
  } else {
    const int row = mt * TC_MT + tid;
    const uint32_t lane_addr = tbase + ((uint32_t)(warp * 32) << 16);
    const int er = (row < a.M) ? a.eA[row] : 0;
    for (int cb = 0; cb < TC_NT; cb += 16) {
      double sum[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) sum[q] = 0.0;
      for (int L = TC_LEVELS + 1; L >= 2; --L) {
        float v[16];
        tmem_ld16(lane_addr + (uint32_t)((L - 2) * TC_NT + cb), v);
        const double w = ldexp(1.0, -14 - 8 * (L - 2));
#pragma unroll
        for (int q = 0; q < 16; ++q) sum[q] = fma((double)v[q], w, sum[q]);
      }
      if (row < a.M) {
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int col = nt * TC_NT + cb + q;
          if (col >= a.N) continue;
          const int ex = er + a.eB[col];
          double* cp = a.C + (long)row * a.crs + (long)col * a.ccs;
          const double prod = ldexp(sum[q], ex);
          *cp = (a.beta == 0.0) ? a.alpha * prod : fma(a.alpha, prod, a.beta * *cp);
          if (a.bound) a.bound[(long)row * a.crs + (long)col * a.ccs] = ldexp(1.0, ex);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tbase, TC_TMEM_COLS);
}

bool g_pairs_set[64] = {false};

int ensure_pairs(int dev) {
  if (dev >= 0 && dev < 64 && g_pairs_set[dev]) return ALPS_OK;
  PairTable t;
  t.n = 0;
  bool seen[TC_S + 2] = {false};
  for (int L = 2; L <= TC_S + 1; ++L)
    for (int sa = 1; sa <= TC_S; ++sa) {
      const int sb = L - sa;
      if (sb < 1 || sb > TC_S) continue;
      t.sa[t.n] = (unsigned char)(sa - 1);
      t.sb[t.n] = (unsigned char)(sb - 1);
      t.lev[t.n] = (unsigned char)L;
      t.first[t.n] = seen[L] ? 0 : 1;
      seen[L] = true;
      t.n++;
    }
  ALPS_CUDA_TRY(cudaMemcpyToSymbol(c_pairs, &t, sizeof(t)));
  ALPS_CUDA_TRY(cudaFuncSetAttribute(k_tc_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * TC_STAGE + 1024));
  if (dev >= 0 && dev < 64) g_pairs_set[dev] = true;
  return ALPS_OK;
}

}  // namespace

// offsets of the workspace parts of an M x N x K product
struct TcLayout {
  size_t As, Bs, eA, eB, err, end;
};
static TcLayout tc_layout(int M, int N, int K) {
  const size_t mt = (M + TC_MT - 1) / TC_MT, nt = (N + TC_NT - 1) / TC_NT, nkc = (K + TC_KC - 1) / TC_KC;
  TcLayout l;
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    size_t at = (off + 255) & ~(size_t)255;
    off = at + bytes;
    return at;
  };
  l.As = carve(mt * nkc * TC_S * TC_A_TILE);
  l.Bs = carve(nt * nkc * TC_S * TC_B_TILE);
  l.eA = carve(mt * TC_MT * sizeof(int));
  l.eB = carve(nt * TC_NT * sizeof(int));
  l.err = carve(sizeof(int));
  l.end = off;
  return l;
}

size_t tc_workspace_bytes(int M, int N, int K) { return tc_layout(M, N, K).end + 256; }

// C = beta C + alpha A B, A (M x K) at A[r*ars + k*aks], B (K x N) at
// B[k*bks + c*bcs], C at C[r*crs + c*ccs]; K <= 256.  kexp (length K, may be
// null): A's column k is scaled by 2^kexp[k] and B's row k by 2^-kexp[k]
// (exact; the product is unchanged).  ws: device workspace of at least
// tc_workspace_bytes(M, N, K).  bound (may be null): per entry the
// fixed-point scale 2^(eA_r + eB_c); the error of the entry is at most
// 10 K 2^-56 times it (times |alpha|).
int tc_product(const double* A, long ars, long aks, const double* B, long bks, long bcs, double* C, long crs,
               long ccs, int M, int N, int K, double alpha, double beta, const int* kexp, void* ws, double* bound,
               cudaStream_t st) {
  if (M <= 0 || N <= 0) return ALPS_OK;
  if (K <= 0 || K > 256) return ALPS_E_INVALID;
  int dev = 0;
  ALPS_CUDA_TRY(cudaGetDevice(&dev));
  int rc = ensure_pairs(dev);
  if (rc) return rc;
  const int mt = (M + TC_MT - 1) / TC_MT, nt = (N + TC_NT - 1) / TC_NT, nkc = (K + TC_KC - 1) / TC_KC;
  unsigned char* w = static_cast<unsigned char*>(ws);
  const TcLayout l = tc_layout(M, N, K);
  __nv_bfloat16* As = reinterpret_cast<__nv_bfloat16*>(w + l.As);
  __nv_bfloat16* Bs = reinterpret_cast<__nv_bfloat16*>(w + l.Bs);
  int* eA = reinterpret_cast<int*>(w + l.eA);
  int* eB = reinterpret_cast<int*>(w + l.eB);
  int* err = reinterpret_cast<int*>(w + l.err);
  ALPS_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
  k_tc_slice<TC_MT><<<(mt * TC_MT * 32 + 255) / 256, 256, 0, st>>>(A, ars, aks, M, K, kexp, 0, nkc, As, eA);
  ALPS_CUDA_TRY(cudaGetLastError());
  // B's role: rows are the output columns c, K along bks
  k_tc_slice<TC_NT><<<(nt * TC_NT * 32 + 255) / 256, 256, 0, st>>>(B, bcs, bks, N, K, kexp, 1, nkc, Bs, eB);
  ALPS_CUDA_TRY(cudaGetLastError());
  TcArgs a;
  a.A = As;
  a.B = Bs;
  a.eA = eA;
  a.eB = eB;
  a.C = C;
  a.crs = crs;
  a.ccs = ccs;
  a.M = M;
  a.N = N;
  a.nkc = nkc;
  a.alpha = alpha;
  a.beta = beta;
  a.err = err;
  a.bound = bound;
  k_tc_gemm<<<dim3(mt, nt), 128, 2 * TC_STAGE + 1024, st>>>(a);
  ALPS_CUDA_TRY(cudaGetLastError());
  return ALPS_OK;
}

void tc_exponents(const void* ws, int M, int N, int K, const int** eA, const int** eB) {
  const TcLayout l = tc_layout(M, N, K);
  *eA = reinterpret_cast<const int*>(static_cast<const unsigned char*>(ws) + l.eA);
  *eB = reinterpret_cast<const int*>(static_cast<const unsigned char*>(ws) + l.eB);
}

// the error word of the last tc_product with this workspace (after sync)
int tc_check(const void* ws, int M, int N, int K) {
  const TcLayout l = tc_layout(M, N, K);
  int e = 0;
  ALPS_CUDA_TRY(cudaMemcpy(&e, static_cast<const unsigned char*>(ws) + l.err, sizeof(int), cudaMemcpyDeviceToHost));
  return e ? ALPS_E_TIMEOUT : ALPS_OK;
}

// ---------------------------------------------------------------------------
// The checked product of the p_perp contraction
// ---------------------------------------------------------------------------
namespace {

// kexp[k] = exponent of max_c |B(k, c)| (0 for a zero row): B's rows to unit
// size, A's columns scaled up by the same power of two
__global__ void k_tc_kexp(const double* __restrict__ B, int K, int N, int* kexp) {
  const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (k >= K) return;
  double mx = 0.0;
  for (int c = lane; c < N; c += 32) mx = fmax(mx, fabs(B[(size_t)k * N + c]));
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) kexp[k] = (mx > 0.0) ? ilogb(mx) : 0;
}

// per entry: M' = sum_k |A~_rk| |B~_kc| in FP32 on the scaled operands
// (A~ = A 2^(kexp - eA_r), B~ = B 2^(-kexp - eB_c), both below 1); where the
// fixed-point bound 10 K 2^-56 exceeds 2^-44 M', the entry is recomputed in
// FP64
__global__ void k_tc_absprep(const double* __restrict__ A, const double* __restrict__ B, int M, int N, int K,
                             const int* __restrict__ kexp, const int* __restrict__ eA,
                             const int* __restrict__ eB, float* Aa, float* Ba) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t na = (size_t)M * K, nb = (size_t)K * N;
  if (t < na) {
    const int r = (int)(t / K), k = (int)(t % K);
    Aa[t] = (float)fabs(ldexp(A[t], kexp[k] - eA[r]));
  } else if (t < na + nb) {
    const size_t u = t - na;
    const int k = (int)(u / N), c = (int)(u % N);
    Ba[u] = (float)fabs(ldexp(B[u], -kexp[k] - eB[c]));
  }
}

// per entry: M' = sum_k |A~||B~| in FP32 from the scaled tables (both
// factors below 1: no overflow); where the fixed-point bound 10 K 2^-56
// exceeds 2^-44 M', the entry is recomputed in FP64
__global__ void k_tc_fixup(const double* __restrict__ A, const double* __restrict__ B, double* C, int M, int N,
                           int K, const float* __restrict__ Aa, const float* __restrict__ Ba, int* nfixed) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y;
  if (c >= N || r >= M) return;
  float m = 0.0f;
  const float* ar = Aa + (size_t)r * K;
  for (int k = 0; k < K; ++k) m = fmaf(ar[k], Ba[(size_t)k * N + c], m);
  // accept when 10 K 2^-56 <= 2^-44 M', i.e. M' >= 10 K 2^-12
  if ((double)m >= 10.0 * K * 0x1p-12) return;
  double s = 0.0;
  for (int k = 0; k < K; ++k) s = fma(A[(size_t)r * K + k], B[(size_t)k * N + c], s);
  C[(size_t)r * N + c] = s;
  atomicAdd(nfixed, 1);
}

}  // namespace

size_t tc_checked_workspace_bytes(int M, int N, int K) {
  return tc_workspace_bytes(M, N, K) + (size_t)M * N * sizeof(double) + (size_t)K * sizeof(int) +
         ((size_t)M * K + (size_t)K * N) * sizeof(float) + 1536;
}

int tc_product_checked(const double* A, const double* B, double* C, int M, int N, int K, void* ws, int* fixed,
                       cudaStream_t st) {
  if (M <= 0 || N <= 0) return ALPS_OK;
  if (K <= 0 || K > 256) return ALPS_E_INVALID;
  unsigned char* w = static_cast<unsigned char*>(ws);
  const size_t base = (tc_workspace_bytes(M, N, K) + 255) & ~(size_t)255;
  double* bound = reinterpret_cast<double*>(w + base);
  int* kexp = reinterpret_cast<int*>(w + ((base + (size_t)M * N * sizeof(double) + 255) & ~(size_t)255));
  int* nfix = kexp + ((K + 63) / 64) * 64;
  float* Aa = reinterpret_cast<float*>(nfix + 64);  // |A~|, then |B~|, FP32
  float* Ba = Aa + (size_t)M * K;
  ALPS_CUDA_TRY(cudaMemsetAsync(nfix, 0, sizeof(int), st));
  k_tc_kexp<<<(K * 32 + 255) / 256, 256, 0, st>>>(B, K, N, kexp);
  ALPS_CUDA_TRY(cudaGetLastError());
  int rc = tc_product(A, K, 1, B, N, 1, C, N, 1, M, N, K, 1.0, 0.0, kexp, w, bound, st);
  if (rc) return rc;
  const int* eA;
  const int* eB;
  tc_exponents(ws, M, N, K, &eA, &eB);
  const size_t nab = (size_t)M * K + (size_t)K * N;
  k_tc_absprep<<<(unsigned)((nab + 255) / 256), 256, 0, st>>>(A, B, M, N, K, kexp, eA, eB, Aa, Ba);
  ALPS_CUDA_TRY(cudaGetLastError());
  k_tc_fixup<<<dim3((N + 127) / 128, M), 128, 0, st>>>(A, B, C, M, N, K, Aa, Ba, nfix);
  ALPS_CUDA_TRY(cudaGetLastError());
  if (fixed) {
    ALPS_CUDA_TRY(cudaMemcpyAsync(fixed, nfix, sizeof(int), cudaMemcpyDeviceToHost, st));
    ALPS_CUDA_TRY(cudaStreamSynchronize(st));
    rc = tc_check(ws, M, N, K);
    if (rc) return rc;
  }
  return ALPS_OK;
}
