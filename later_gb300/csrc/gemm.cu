// Tensor-core GEMM for sm_103a: TMA-fed, tcgen05.mma with the accumulator in
// TMEM, FP16 / BF16 operands and FP32 accumulation.
//
//   D = alpha * op(A) * op(B) + beta * C,   column-major, op = N or T.
//
// This is the kernel behind every trailing update of the recursion drivers.
// In the reference those are cublasGemmEx calls on FP16 copies produced by
// separate s2h passes (QR/later_rgsqrf.cu:43-56, QR/later_rhouqr.cu:111-134,
// BLAS/later_rsyrk.cu:38-65, BLAS/later_rtrsm.cu:101-112,150-160,
// BLAS/later_rtrmm.cu:40-51). Here the epilogue writes the FP32 result and,
// when asked, its 16-bit copy in the same pass, so the next GEMM of the
// recursion reads its operand without a conversion pass.
//
// Two kernels share the stage layout and MMA issue:
// tc_gemm_kernel (one CTA = one 128 x BN output tile, or one K-slice of it):
//   warp 0 / lane 0 : TMA producer, STAGES-deep ring of 64-wide K blocks
//   warp 1 / lane 0 : MMA issuer (tcgen05.mma, M=128, N=BN, K=16 steps);
//                     warp 1 also owns the TMEM allocation
//   warps 2-7       : prefetch the tile's C block into L2 during the mainloop
//   warps 0-7       : epilogue, two warps per TMEM lane quarter (32 rows),
//                     alternate 32-column chunks
//   Split-K: CTAs of one tile write FP32 partial tiles; splitk_reduce_kernel
//   sums them in split order in a fixed tree, so results are deterministic.
// tc_gemm_persistent_kernel (the TN / NN trailing updates without split-K):
//   one CTA per SM walks the tiles; producer and MMA issuer run across tiles,
//   two TMEM accumulators let warps 4-11 run one tile's epilogue while the next
//   tile's MMAs run.
// Tiles are visited in groups of 16 tile rows, so concurrent CTAs share A and
// B panels through L2.
// SPLIT3: A = Ah + Al/2048, B = Bh + Bl/2048 (FP16); three products go to two
// TMEM accumulators, D = acc0 + acc1/2048. SPLIT2: A = Ah + Al/2048, B = Bh;
// two products (Ah.Bh and Al.Bh) into two accumulators, combined the same way.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdlib>
#include <mutex>

#include "ptx.cuh"
#include "runtime.cuh"

namespace later {

namespace {

constexpr int BM = 128;
constexpr int BK = 64;
// Warp 0 lane 0 issues the TMA loads, warp 1 lane 0 the MMAs (warp 1 owns the
// TMEM allocation), warps 2..7 prefetch C into L2; then all eight warps run the
// epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (its lane quarter) and
// the 32-column chunks c0 = 32 (w / 4), + 64, ... of the tile.
constexpr int kGemmThreads = 256;
constexpr float kLoScale = 2048.f;       // SPLIT3 lo operands are stored scaled by 2^11
constexpr float kLoScaleInv = 1.f / 2048.f;

struct GemmArgs {
  int M, N, K;
  int kb_total, kb_per_split, splits;
  int tiles_m, tiles_n;
  float alpha, beta;
  const float* C;
  int64_t ldc;
  float* D;
  int64_t ldd;
  void* Dh;
  void* Dl;
  int64_t ldh;
  int out_mode;  // 0 fp16, 1 bf16, 2 split3 (hi/lo fp16)
  int lower, diag;
  int shadow_acc;
  int round_prod;
  int ab_bf16;
  float* partial;
  int* counters;
  int* status;
  long long budget;
};

// Output tile of linear index t, in groups of kGroupM tile rows: inside a
// group the row index varies fastest, so the CTAs resident at one time cover
// about kGroupM x (CTAs / kGroupM) tiles and share their A row panels and B
// column panels through L2 instead of each streaming its own A panel from HBM.
constexpr int kGroupM = 16;
__device__ __forceinline__ void tile_coords(int t, int tiles_m, int tiles_n, int* tm, int* tn) {
  const int per_group = kGroupM * tiles_n;
  const int first_m = (t / per_group) * kGroupM;
  const int rows = min(tiles_m - first_m, kGroupM);
  const int r = t % per_group;
  *tm = first_m + r % rows;
  *tn = r / rows;
}

__device__ __forceinline__ void store16(void* base, int64_t idx, float v, int bf16) {
  if (bf16)
    reinterpret_cast<__nv_bfloat16*>(base)[idx] = __float2bfloat16_rn(v);
  else
    reinterpret_cast<__half*>(base)[idx] = __float2half_rn(v);
}

// Epilogue of one output element: D = alpha*acc + beta*C, plus the 16-bit copy.
// `c` is the already-loaded C element (ignored when beta == 0).
__device__ __forceinline__ void epilogue_store_c(const GemmArgs& p, int row, int col, float acc, float c) {
  if (row >= p.M || col >= p.N) return;
  if (p.lower && row < col + p.diag) return;
  float prod = p.alpha * acc;
  if (p.round_prod) prod = __half2float(__float2half_rn(prod));
  float v = prod;
  if (p.beta != 0.f) v += p.beta * c;
  p.D[row + static_cast<int64_t>(col) * p.ldd] = v;
  if (p.Dh) {
    if (p.shadow_acc) v = prod;
    const int64_t hidx = row + static_cast<int64_t>(col) * p.ldh;
    if (p.out_mode == 1) {
      store16(p.Dh, hidx, v, 1);
    } else {
      if (fabsf(v) > 65504.f) report(p.status, DEV_RANGE);
      const __half h = __float2half_rn(v);
      reinterpret_cast<__half*>(p.Dh)[hidx] = h;
      if (p.out_mode == 2)
        reinterpret_cast<__half*>(p.Dl)[hidx] = __float2half_rn((v - __half2float(h)) * kLoScale);
    }
  }
}

// SPL: 0 one product; 1 A split (hi.hi into accumulator 0, lo.hi into 1);
// 2 both split, SPLIT3 (hi.hi into 0, hi.lo + lo.hi into 1).
// Epilogue of 32 interior elements of one row (columns col0 .. col0 + 31, all
// inside the output, no triangle): the same arithmetic as epilogue_store_c
// with the mode tests hoisted out of the element loop.
__device__ __forceinline__ void epilogue_chunk(const GemmArgs& p, int row, int col0, const float (&acc)[32],
                                               const float (&c)[32]) {
  float prod[32], val[32];
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    prod[j] = p.alpha * acc[j];
    if (p.round_prod) prod[j] = __half2float(__float2half_rn(prod[j]));
    val[j] = p.beta != 0.f ? prod[j] + p.beta * c[j] : prod[j];
  }
  float* d = p.D + row + static_cast<int64_t>(col0) * p.ldd;
#pragma unroll
  for (int j = 0; j < 32; ++j) d[j * p.ldd] = val[j];
  if (!p.Dh) return;
  const float* src = p.shadow_acc ? prod : val;
  const int64_t h0 = row + static_cast<int64_t>(col0) * p.ldh;
  if (p.out_mode == 1) {
    __nv_bfloat16* h = reinterpret_cast<__nv_bfloat16*>(p.Dh) + h0;
#pragma unroll
    for (int j = 0; j < 32; ++j) h[j * p.ldh] = __float2bfloat16_rn(src[j]);
    return;
  }
  __half* h = reinterpret_cast<__half*>(p.Dh) + h0;
  bool big = false;
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    big |= fabsf(src[j]) > 65504.f;
    h[j * p.ldh] = __float2half_rn(src[j]);
  }
  if (big) report(p.status, DEV_RANGE);
  if (p.out_mode == 2) {
    __half* l = reinterpret_cast<__half*>(p.Dl) + h0;
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const float hv = __half2float(__float2half_rn(src[j]));
      l[j * p.ldh] = __float2half_rn((src[j] - hv) * kLoScale);
    }
  }
}

template <int BN, bool A_MN, bool B_MN, int SPL, int STAGES>
struct Cfg {
  static constexpr int A_BYTES = BM * BK * 2;  // 16 KB
  static constexpr int B_BYTES = BN * BK * 2;
  static constexpr int A_OPS = SPL ? 2 : 1;
  static constexpr int B_OPS = SPL == 2 ? 2 : 1;
  static constexpr int STAGE_BYTES = A_OPS * A_BYTES + B_OPS * B_BYTES;
  static constexpr int TMEM_COLS = SPL ? 2 * BN : BN;
  static constexpr int SMEM = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
};

template <int BN, bool A_MN, bool B_MN, int SPL, int STAGES>
__global__ void __launch_bounds__(kGemmThreads, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   const __grid_constant__ CUtensorMap tmAl, const __grid_constant__ CUtensorMap tmBl,
                   const GemmArgs p) {
  using C_ = Cfg<BN, A_MN, B_MN, SPL, STAGES>;
  static_assert(C_::TMEM_COLS >= 32 && C_::TMEM_COLS <= 512, "tmem");
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * C_::STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* done = empty + STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  volatile int* last_flag = abort_flag + 1;

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  int tile_m, tile_n;
  tile_coords(blockIdx.x, p.tiles_m, p.tiles_n, &tile_m, &tile_n);
  const int split = blockIdx.y;
  const int m0 = tile_m * BM;
  const int n0 = tile_n * BN;
  const int kb0 = split * p.kb_per_split;
  const int kb1 = min(kb0 + p.kb_per_split, p.kb_total);
  const int nkb = kb1 - kb0;
  // Lower-triangular output (SYRK): a tile entirely above the diagonal has no work.
  if (p.lower && m0 + BM - 1 < n0 + p.diag) {
    griddep_wait();
    return;
  }

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    *last_flag = 0;
    fence_barrier_init();
  }
  if (warp == 1) tmem_alloc(tmem_slot, C_::TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  griddep_wait();  // operands and C are written by the previous kernel in the stream
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // ------------------------------------------------------- producer
      tma_prefetch_desc(&tmA);
      tma_prefetch_desc(&tmB);
      if (SPL) tma_prefetch_desc(&tmAl);
      if (SPL == 2) tma_prefetch_desc(&tmBl);
      int issued = 0;
      for (int i = 0; i < nkb; ++i) {
        const int s = i % STAGES;
        const uint32_t ph = (i / STAGES) & 1;
        if (i >= STAGES && !mbar_wait(&empty[s], ph ^ 1, p.budget)) {
          *abort_flag = 1;
          break;
        }
        if (*abort_flag) break;
        uint8_t* sa = smem + s * C_::STAGE_BYTES;
        uint8_t* sb = sa + C_::A_OPS * C_::A_BYTES;
        const int k0 = (kb0 + i) * BK;
        mbar_arrive_expect_tx(&full[s], C_::STAGE_BYTES);
#pragma unroll
        for (int op = 0; op < C_::A_OPS; ++op) {
          const CUtensorMap* ma = op ? &tmAl : &tmA;
          uint8_t* da = sa + op * C_::A_BYTES;
          if (A_MN) {
            tma_load_2d(da, ma, &full[s], m0, k0);
            tma_load_2d(da + BK * 128, ma, &full[s], m0 + 64, k0);
          } else {
            tma_load_2d(da, ma, &full[s], k0, m0);
          }
        }
#pragma unroll
        for (int op = 0; op < C_::B_OPS; ++op) {
          const CUtensorMap* mb = op ? &tmBl : &tmB;
          uint8_t* db = sb + op * C_::B_BYTES;
          if (B_MN) {
#pragma unroll
            for (int c = 0; c < BN / 64; ++c) tma_load_2d(db + c * BK * 128, mb, &full[s], n0 + 64 * c, k0);
          } else {
            tma_load_2d(db, mb, &full[s], k0, n0);
          }
        }
        ++issued;
      }
      // Drain: every issued load must land before the CTA may exit.
      for (int j = (issued > STAGES ? issued - STAGES : 0); j < issued; ++j)
        mbar_wait(&full[j % STAGES], (j / STAGES) & 1, kDrainBudgetCycles);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ------------------------------------------------------- MMA issuer
      const uint32_t idesc = idesc_f16(BM, BN, p.ab_bf16, A_MN ? 1 : 0, B_MN ? 1 : 0);
      for (int i = 0; i < nkb; ++i) {
        const int s = i % STAGES;
        const uint32_t ph = (i / STAGES) & 1;
        if (!mbar_wait(&full[s], ph, p.budget)) {
          *abort_flag = 1;
          break;
        }
        if (*abort_flag) break;
        tc_fence_after();
        const uint32_t sa = smem_u32(smem + s * C_::STAGE_BYTES);
        const uint32_t sb = sa + C_::A_OPS * C_::A_BYTES;
#pragma unroll
        for (int k = 0; k < BK / 16; ++k) {
          // A: K-major -> advance 32 B within the swizzled row; MN-major -> 16 K-rows.
          const uint32_t a_off = A_MN ? k * 16 * 128 : k * 32;
          const uint32_t b_off = B_MN ? k * 16 * 128 : k * 32;
          const uint64_t ad = smem_desc_sw128(sa + a_off, A_MN ? BK * 128 : 16, 1024);
          const uint64_t bd = smem_desc_sw128(sb + b_off, B_MN ? BK * 128 : 16, 1024);
          const uint32_t acc = (i > 0 || k > 0) ? 1u : 0u;
          tc_mma_f16(tmem, ad, bd, idesc, acc);
          if (SPL == 2) {
            const uint64_t adl = smem_desc_sw128(sa + C_::A_BYTES + a_off, A_MN ? BK * 128 : 16, 1024);
            const uint64_t bdl = smem_desc_sw128(sb + C_::B_BYTES + b_off, B_MN ? BK * 128 : 16, 1024);
            tc_mma_f16(tmem + BN, ad, bdl, idesc, acc);
            tc_mma_f16(tmem + BN, adl, bd, idesc, 1u);
          } else if (SPL == 1) {
            const uint64_t adl = smem_desc_sw128(sa + C_::A_BYTES + a_off, A_MN ? BK * 128 : 16, 1024);
            tc_mma_f16(tmem + BN, adl, bd, idesc, acc);
          }
        }
        tc_commit(&empty[s]);
      }
      tc_commit(done);  // arrives once every MMA above has completed
    }
  } else if (p.beta != 0.f && p.splits == 1) {
    // Warps 2-3 are idle during the mainloop: pull this tile's C block into L2
    // so that the epilogue's reads of it hit L2 rather than HBM.
    const int rows = min(BM, p.M - m0), ncols = min(BN, p.N - n0);
    if (rows > 0 && ncols > 0) {
      const int lines = (rows + 31) / 32;  // 128-byte lines of 32 floats per column
      for (int e = threadIdx.x - 64; e < ncols * lines; e += kGemmThreads - 64) {
        const int c = e / lines, l = e % lines;
        const float* addr = p.C + m0 + 32 * l + static_cast<int64_t>(n0 + c) * p.ldc;
        asm volatile("prefetch.global.L2 [%0];" ::"l"(addr));
      }
    }
  }
  __syncwarp();

  // --------------------------------------------------------------- epilogue
  const bool drained = mbar_wait(done, 0, kDrainBudgetCycles);
  tc_fence_after();
  griddep_launch();  // the next kernel's CTAs may be scheduled while this epilogue runs
  const bool ok = drained && (*abort_flag == 0) && nkb > 0;
  if (!ok && threadIdx.x == 0) report(p.status, DEV_TIMEOUT);

  const int quarter = warp & 3, half = warp >> 2;
  const int r = quarter * 32 + lane;  // tile row == TMEM lane
  const int row = m0 + r;
  const uint32_t t_row = tmem + (static_cast<uint32_t>(quarter * 32) << 16);
  // Split-K: this CTA's FP32 partial tile, [col][row], reduced by splitk_reduce_kernel.
  float* mine = p.splits > 1 ? p.partial + (static_cast<int64_t>(blockIdx.x) * p.splits + split) * (BM * BN)
                             : nullptr;
  // C values of a 32-column chunk are loaded one chunk ahead of the chunk's
  // stores. C and D may alias: each element is read and written by the same
  // thread, and a chunk's C is read before any of its D stores.
  const bool rd = (p.beta != 0.f) && row < p.M && ok && !mine;
  float cv[32];
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    const int col = n0 + 32 * half + j;
    cv[j] = (rd && 32 * half < BN && col < p.N) ? p.C[row + static_cast<int64_t>(col) * p.ldc] : 0.f;
  }
#pragma unroll 1
  for (int c0 = 32 * half; c0 < BN; c0 += 64) {
    float v[32];
    tmem_ld_32x32b_x32(t_row + c0, v);
    if (SPL) {
      float w[32];
      tmem_ld_32x32b_x32(t_row + BN + c0, w);
#pragma unroll
      for (int j = 0; j < 32; ++j) v[j] += w[j] * kLoScaleInv;
    }
    if (mine) {
#pragma unroll
      for (int j = 0; j < 32; ++j) __stcg(&mine[(c0 + j) * BM + r], ok ? v[j] : 0.f);
    } else if (ok) {
      float cn[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int col = n0 + c0 + 64 + j;
        cn[j] = (rd && c0 + 64 < BN && col < p.N) ? p.C[row + static_cast<int64_t>(col) * p.ldc] : 0.f;
      }
      if (row < p.M && n0 + c0 + 32 <= p.N && !p.lower) {
        epilogue_chunk(p, row, n0 + c0, v, cv);
      } else {
#pragma unroll
        for (int j = 0; j < 32; ++j) epilogue_store_c(p, row, n0 + c0 + j, v[j], cv[j]);
      }
#pragma unroll
      for (int j = 0; j < 32; ++j) cv[j] = cn[j];
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) tmem_dealloc(tmem, C_::TMEM_COLS);
}

// Deterministic split-K reduction: 256 threads = 32 rows x 8 slices; slice j
// sums partials j, j+8, ... in order, then the 8 slice sums are combined in a
// fixed tree. One block covers 32 rows x 4 columns of one tile.
template <int BN>
__global__ void __launch_bounds__(256) splitk_reduce_kernel(const GemmArgs p) {
  __shared__ float part[8][4][33];
  griddep_wait();
  const int tiles_per_row_groups = (BM / 32) * (BN / 4);
  const int tile = blockIdx.x / tiles_per_row_groups;
  const int rem = blockIdx.x % tiles_per_row_groups;
  const int rg = rem % (BM / 32);
  const int cg = rem / (BM / 32);
  int tile_m, tile_n;
  tile_coords(tile, p.tiles_m, p.tiles_n, &tile_m, &tile_n);
  const int r = rg * 32 + threadIdx.x % 32;
  const int j = threadIdx.x / 32;
  const float* base = p.partial + static_cast<int64_t>(tile) * p.splits * (BM * BN);
#pragma unroll
  for (int cc = 0; cc < 4; ++cc) {
    const int c = cg * 4 + cc;
    float acc = 0.f;
#pragma unroll 8
    for (int s = j; s < p.splits; s += 8) acc += __ldcg(&base[static_cast<int64_t>(s) * (BM * BN) + c * BM + r]);
    part[j][cc][threadIdx.x % 32] = acc;
  }
  __syncthreads();
  if (j < 4) {
    const int cc = j;
    const int l = threadIdx.x % 32;
    const float v = ((part[0][cc][l] + part[1][cc][l]) + (part[2][cc][l] + part[3][cc][l])) +
                    ((part[4][cc][l] + part[5][cc][l]) + (part[6][cc][l] + part[7][cc][l]));
    const int row = tile_m * BM + r, col = tile_n * BN + cg * 4 + cc;
    const float c = (p.beta != 0.f && row < p.M && col < p.N) ? p.C[row + static_cast<int64_t>(col) * p.ldc] : 0.f;
    epilogue_store_c(p, row, col, v, c);
  }
}

// ------------------------------------------------------- persistent kernel
// One CTA per SM walks the output tiles t = blockIdx.x, + gridDim.x, ... (the
// grouped order of tile_coords), without split-K. Warp 0 lane 0 issues the TMA
// loads and warp 1 lane 0 the MMAs continuously across tiles: the stage ring's
// index and phase follow one k-block counter over all of the CTA's tiles.
// Accumulators: NACC TMEM buffers of ACC_COLS columns; the MMA of tile i goes
// to buffer i % NACC once the epilogue has drained that buffer's previous use
// (tmem_empty), and signals tmem_full when its MMAs complete. Warps 4..11 run
// the epilogue (two warps per TMEM lane quarter, alternate 32-column chunks),
// so with NACC = 2 the epilogue of one tile overlaps the mainloop of the next,
// and the loads of the next tile overlap the epilogue in any case. Before
// waiting for a tile they prefetch its C block into L2. Every wait is bounded;
// on a timeout the CTA sets DEV_TIMEOUT, stops issuing, drains its loads and
// MMAs, and returns.
constexpr int kPersistThreads = 384;
constexpr int kEpiWarp0 = 4;  // warps 4 .. 11
constexpr int kEpiThreads = 256;

template <int BN, bool A_MN, bool B_MN, int SPL, int STAGES, int NACC>
struct PCfg {
  using Base = Cfg<BN, A_MN, B_MN, SPL, STAGES>;
  static_assert(Base::TMEM_COLS > 0 && Base::SMEM > 0, "stage layout shared with the one-tile kernel");
  static constexpr int ACC_COLS = SPL ? 2 * BN : BN;
  static constexpr int TMEM_COLS = NACC * ACC_COLS;
  static constexpr int SMEM = STAGES * Base::STAGE_BYTES + 1024 + 256;
};

template <int BN, bool A_MN, bool B_MN, int SPL, int STAGES, int NACC>
__global__ void __launch_bounds__(kPersistThreads, 1)
    tc_gemm_persistent_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                              const __grid_constant__ CUtensorMap tmAl, const __grid_constant__ CUtensorMap tmBl,
                              const GemmArgs p) {
  using C_ = Cfg<BN, A_MN, B_MN, SPL, STAGES>;
  using P_ = PCfg<BN, A_MN, B_MN, SPL, STAGES, NACC>;
  static_assert(P_::TMEM_COLS == 32 || P_::TMEM_COLS == 64 || P_::TMEM_COLS == 128 || P_::TMEM_COLS == 256 ||
                    P_::TMEM_COLS == 512,
                "tmem allocation must be a power of two in [32, 512]");
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * C_::STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* tfull = empty + STAGES;
  uint64_t* tempty = tfull + NACC;
  uint64_t* done = tempty + NACC;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int ntiles = p.tiles_m * p.tiles_n;
  const int nkb = p.kb_total;
  // Same skip rule in every role: a lower-triangular output's tiles entirely above the diagonal.
  auto skip = [&](int t) {
    int tm, tn;
    tile_coords(t, p.tiles_m, p.tiles_n, &tm, &tn);
    return p.lower && tm * BM + BM - 1 < tn * BN + p.diag;
  };

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int a = 0; a < NACC; ++a) {
      mbar_init(&tfull[a], 1);
      mbar_init(&tempty[a], kEpiThreads);
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    fence_barrier_init();
  }
  if (warp == 1) tmem_alloc(tmem_slot, P_::TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  griddep_wait();  // operands and C are written by the previous kernel in the stream
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // ------------------------------------------------------- producer
      tma_prefetch_desc(&tmA);
      tma_prefetch_desc(&tmB);
      if (SPL) tma_prefetch_desc(&tmAl);
      if (SPL == 2) tma_prefetch_desc(&tmBl);
      uint32_t g = 0;
      for (int t = blockIdx.x; t < ntiles && !*abort_flag; t += gridDim.x) {
        if (skip(t)) continue;
        int tm, tn;
        tile_coords(t, p.tiles_m, p.tiles_n, &tm, &tn);
        const int m0 = tm * BM, n0 = tn * BN;
        for (int i = 0; i < nkb; ++i, ++g) {
          const int s = g % STAGES;
          const uint32_t ph = (g / STAGES) & 1;
          if (g >= STAGES && !mbar_wait(&empty[s], ph ^ 1, p.budget)) {
            *abort_flag = 1;
            break;
          }
          if (*abort_flag) break;
          uint8_t* sa = smem + s * C_::STAGE_BYTES;
          uint8_t* sb = sa + C_::A_OPS * C_::A_BYTES;
          const int k0 = i * BK;
          mbar_arrive_expect_tx(&full[s], C_::STAGE_BYTES);
#pragma unroll
          for (int op = 0; op < C_::A_OPS; ++op) {
            const CUtensorMap* ma = op ? &tmAl : &tmA;
            uint8_t* da = sa + op * C_::A_BYTES;
            if (A_MN) {
              tma_load_2d(da, ma, &full[s], m0, k0);
              tma_load_2d(da + BK * 128, ma, &full[s], m0 + 64, k0);
            } else {
              tma_load_2d(da, ma, &full[s], k0, m0);
            }
          }
#pragma unroll
          for (int op = 0; op < C_::B_OPS; ++op) {
            const CUtensorMap* mb = op ? &tmBl : &tmB;
            uint8_t* db = sb + op * C_::B_BYTES;
            if (B_MN) {
#pragma unroll
              for (int c = 0; c < BN / 64; ++c) tma_load_2d(db + c * BK * 128, mb, &full[s], n0 + 64 * c, k0);
            } else {
              tma_load_2d(db, mb, &full[s], k0, n0);
            }
          }
        }
      }
      griddep_launch();  // every load of this CTA is issued: the next kernel may be scheduled
      // Drain: every issued load must land before the CTA may exit.
      for (uint32_t j = (g > STAGES ? g - STAGES : 0); j < g; ++j)
        mbar_wait(&full[j % STAGES], (j / STAGES) & 1, kDrainBudgetCycles);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ------------------------------------------------------- MMA issuer
      const uint32_t idesc = idesc_f16(BM, BN, p.ab_bf16, A_MN ? 1 : 0, B_MN ? 1 : 0);
      uint32_t g = 0;
      int lt = 0;
      for (int t = blockIdx.x; t < ntiles && !*abort_flag; t += gridDim.x) {
        if (skip(t)) continue;
        const int a = lt % NACC, use = lt / NACC;
        if (use > 0 && !mbar_wait(&tempty[a], (use - 1) & 1, p.budget)) {
          *abort_flag = 1;
          break;
        }
        tc_fence_after();
        const uint32_t acc_base = tmem + a * P_::ACC_COLS;
        for (int i = 0; i < nkb; ++i, ++g) {
          const int s = g % STAGES;
          const uint32_t ph = (g / STAGES) & 1;
          if (!mbar_wait(&full[s], ph, p.budget)) {
            *abort_flag = 1;
            break;
          }
          if (*abort_flag) break;
          tc_fence_after();
          const uint32_t sa = smem_u32(smem + s * C_::STAGE_BYTES);
          const uint32_t sb = sa + C_::A_OPS * C_::A_BYTES;
#pragma unroll
          for (int k = 0; k < BK / 16; ++k) {
            const uint32_t a_off = A_MN ? k * 16 * 128 : k * 32;
            const uint32_t b_off = B_MN ? k * 16 * 128 : k * 32;
            const uint64_t ad = smem_desc_sw128(sa + a_off, A_MN ? BK * 128 : 16, 1024);
            const uint64_t bd = smem_desc_sw128(sb + b_off, B_MN ? BK * 128 : 16, 1024);
            const uint32_t acc = (i > 0 || k > 0) ? 1u : 0u;
            tc_mma_f16(acc_base, ad, bd, idesc, acc);
            if (SPL == 2) {
              const uint64_t adl = smem_desc_sw128(sa + C_::A_BYTES + a_off, A_MN ? BK * 128 : 16, 1024);
              const uint64_t bdl = smem_desc_sw128(sb + C_::B_BYTES + b_off, B_MN ? BK * 128 : 16, 1024);
              tc_mma_f16(acc_base + BN, ad, bdl, idesc, acc);
              tc_mma_f16(acc_base + BN, adl, bd, idesc, 1u);
            } else if (SPL == 1) {
              const uint64_t adl = smem_desc_sw128(sa + C_::A_BYTES + a_off, A_MN ? BK * 128 : 16, 1024);
              tc_mma_f16(acc_base + BN, adl, bd, idesc, acc);
            }
          }
          tc_commit(&empty[s]);
        }
        if (*abort_flag) break;
        tc_commit(&tfull[a]);  // arrives once this tile's MMAs have completed
        ++lt;
      }
      tc_commit(done);  // every MMA issued above has completed when this arrives
      mbar_wait(done, 0, kDrainBudgetCycles);
    }
  } else if (warp >= kEpiWarp0) {
    // ------------------------------------------------------- epilogue
    const int ew = warp - kEpiWarp0;
    const int quarter = warp & 3, half = ew >> 2;  // TMEM lanes 32 (warp % 4) .. + 31
    const int r = quarter * 32 + lane;
    int lt = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      if (skip(t)) continue;
      int tm, tn;
      tile_coords(t, p.tiles_m, p.tiles_n, &tm, &tn);
      const int m0 = tm * BM, n0 = tn * BN;
      // this tile's C block into L2 while its MMAs run
      if (p.beta != 0.f) {
        const int rows = min(BM, p.M - m0), ncols = min(BN, p.N - n0);
        const int lines = (rows + 31) / 32;
        for (int e = threadIdx.x - kEpiWarp0 * 32; e < ncols * lines; e += kEpiThreads) {
          const int c = e / lines, l = e % lines;
          asm volatile("prefetch.global.L2 [%0];" ::"l"(p.C + m0 + 32 * l + static_cast<int64_t>(n0 + c) * p.ldc));
        }
      }
      const int a = lt % NACC, use = lt / NACC;
      if (!mbar_wait(&tfull[a], use & 1, p.budget)) {
        if (threadIdx.x == kEpiWarp0 * 32) report(p.status, DEV_TIMEOUT);
        *abort_flag = 1;
        break;
      }
      tc_fence_after();
      const int row = m0 + r;
      const uint32_t t_row = tmem + a * P_::ACC_COLS + (static_cast<uint32_t>(quarter * 32) << 16);
      const bool rd = (p.beta != 0.f) && row < p.M;
      float cv[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int col = n0 + 32 * half + j;
        cv[j] = (rd && 32 * half < BN && col < p.N) ? p.C[row + static_cast<int64_t>(col) * p.ldc] : 0.f;
      }
#pragma unroll 1
      for (int c0 = 32 * half; c0 < BN; c0 += 64) {
        float v[32];
        tmem_ld_32x32b_x32(t_row + c0, v);
        if (SPL) {
          float w[32];
          tmem_ld_32x32b_x32(t_row + BN + c0, w);
#pragma unroll
          for (int j = 0; j < 32; ++j) v[j] += w[j] * kLoScaleInv;
        }
        float cn[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int col = n0 + c0 + 64 + j;
          cn[j] = (rd && c0 + 64 < BN && col < p.N) ? p.C[row + static_cast<int64_t>(col) * p.ldc] : 0.f;
        }
        if (row < p.M && n0 + c0 + 32 <= p.N && !p.lower) {
          epilogue_chunk(p, row, n0 + c0, v, cv);
        } else {
#pragma unroll
          for (int j = 0; j < 32; ++j) epilogue_store_c(p, row, n0 + c0 + j, v[j], cv[j]);
        }
#pragma unroll
        for (int j = 0; j < 32; ++j) cv[j] = cn[j];
      }
      tc_fence_before();
      mbar_arrive(&tempty[a]);  // this thread's reads of buffer a are complete
      ++lt;
    }
  }
  __syncwarp();
  tc_fence_before();
  __syncthreads();
  if (warp == 1) tmem_dealloc(tmem, P_::TMEM_COLS);
}

template <int BN, bool A_MN, bool B_MN, int SPL, int STAGES, int NACC>
later_status_t launch_persistent(const CUtensorMap& a, const CUtensorMap& b, const CUtensorMap& al,
                                 const CUtensorMap& bl, const GemmArgs& args, int ctas, cudaStream_t st) {
  using P_ = PCfg<BN, A_MN, B_MN, SPL, STAGES, NACC>;
  static_assert(P_::SMEM <= 227 * 1024, "shared memory");
  auto kern = tc_gemm_persistent_kernel<BN, A_MN, B_MN, SPL, STAGES, NACC>;
  static bool attr_done[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && !attr_done[dev]) {
    LATER_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, P_::SMEM));
    attr_done[dev] = true;
  }
  LATER_CHECK_CUDA(launch_pdl(kern, dim3(ctas), dim3(kPersistThreads), P_::SMEM, st, a, b, al, bl, args));
  note_launch();
  return LATER_OK;
}

// The trailing-update shapes of rgsqrf: TN (R12 = Q1^T A2) and NN (A2 -= Q1 R12).
template <int BN, int SPL, int STAGES, int NACC>
later_status_t launch_persistent_ab(bool a_mn, bool b_mn, const CUtensorMap& a, const CUtensorMap& b,
                                    const CUtensorMap& al, const CUtensorMap& bl, const GemmArgs& args, int ctas,
                                    cudaStream_t st) {
  if (b_mn) return LATER_ERR_NOT_SUPPORTED;
  if (a_mn) return launch_persistent<BN, true, false, SPL, STAGES, NACC>(a, b, al, bl, args, ctas, st);
  return launch_persistent<BN, false, false, SPL, STAGES, NACC>(a, b, al, bl, args, ctas, st);
}

// ------------------------------------------------------------------- host
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void* f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  });
  return fn;
}

template <int BN, bool A_MN, bool B_MN, int SPL, int STAGES>
later_status_t launch_cfg(const CUtensorMap& a, const CUtensorMap& b, const CUtensorMap& al,
                          const CUtensorMap& bl, const GemmArgs& args, dim3 grid, cudaStream_t st) {
  using C_ = Cfg<BN, A_MN, B_MN, SPL, STAGES>;
  static_assert(C_::SMEM <= 227 * 1024, "shared memory");
  auto kern = tc_gemm_kernel<BN, A_MN, B_MN, SPL, STAGES>;
  static bool attr_done[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && !attr_done[dev]) {
    LATER_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C_::SMEM));
    attr_done[dev] = true;
  }
  LATER_CHECK_CUDA(launch_pdl(kern, grid, dim3(kGemmThreads), C_::SMEM, st, a, b, al, bl, args));
  note_launch();
  if (args.splits > 1) {
    const int blocks = static_cast<int>(grid.x) * (BM / 32) * (BN / 4);
    LATER_CHECK_CUDA(launch_pdl(splitk_reduce_kernel<BN>, dim3(blocks), dim3(256), 0, st, args));
    note_launch();
  }
  return LATER_OK;
}

template <int BN, int SPL, int STAGES>
later_status_t launch_bn(bool a_mn, bool b_mn, const CUtensorMap& a, const CUtensorMap& b,
                         const CUtensorMap& al, const CUtensorMap& bl, const GemmArgs& args, dim3 grid,
                         cudaStream_t st) {
  if (!a_mn && !b_mn) return launch_cfg<BN, false, false, SPL, STAGES>(a, b, al, bl, args, grid, st);
  if (a_mn && !b_mn) return launch_cfg<BN, true, false, SPL, STAGES>(a, b, al, bl, args, grid, st);
  if (a_mn && b_mn) return launch_cfg<BN, true, true, SPL, STAGES>(a, b, al, bl, args, grid, st);
  return launch_cfg<BN, false, true, SPL, STAGES>(a, b, al, bl, args, grid, st);
}

}  // namespace

bool make_map16(CUtensorMap* map, const void* base, uint64_t rows, uint64_t cols, uint64_t ld,
                uint32_t box_rows, uint32_t box_cols, bool bf16) {
  auto fn = encode_fn();
  if (!fn) return false;
  if ((reinterpret_cast<uintptr_t>(base) & 15) != 0 || (ld * 2) % 16 != 0) return false;
  cuuint64_t dims[2] = {rows, cols};
  cuuint64_t strides[1] = {ld * 2};
  cuuint32_t box[2] = {box_rows, box_cols};
  cuuint32_t es[2] = {1, 1};
  CUresult r = fn(map, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2,
                  const_cast<void*>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// The persistent kernel is used unless LATER_GEMM_PERSISTENT=0 (kept for A/B timing).
bool persistent_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("LATER_GEMM_PERSISTENT");
    return !(e && e[0] == '0');
  }();
  return on;
}

later_status_t tc_gemm(const GemmCall& g, const Scratch& s, cudaStream_t st, long long budget) {
  if (g.M <= 0 || g.N <= 0) return LATER_OK;
  if (g.K <= 0) return LATER_ERR_INVALID_ARG;
  const bool a_mn = (g.ta == 'N' || g.ta == 'n');
  const bool b_mn = (g.tb == 'T' || g.tb == 't');
  const bool split3 = (g.prec == LATER_PREC_SPLIT3);
  const bool split_a = (g.prec == LATER_PREC_SPLIT2);  // A = hi + lo, B = hi: two products
  const bool bf16 = (g.prec == LATER_PREC_BF16);
  if (g.prec < LATER_PREC_FP16 || g.prec > LATER_PREC_SPLIT2) return LATER_ERR_INVALID_ARG;
  if (split3 && (!g.A.lo || !g.B.lo)) return LATER_ERR_INVALID_ARG;
  if (split_a && (!g.A.lo || !a_mn || b_mn)) return LATER_ERR_INVALID_ARG;  // the A2 -= Q1 R12 shape only
  if (g.out.Dh && g.out_prec == LATER_PREC_SPLIT3 && !g.out.Dl) return LATER_ERR_INVALID_ARG;

  // Tile width: the widest of 256 / 128 / 64 that still gives the GPU enough tiles.
  const int nsm = num_sms();
  const int tiles_m = static_cast<int>((g.M + BM - 1) / BM);
  int BN = 128;
  if (!split3 && static_cast<int64_t>(tiles_m) * ((g.N + 255) / 256) >= nsm) BN = 256;
  if (g.N <= 64) BN = 64;
  const int tiles_n = (g.N + BN - 1) / BN;
  const int tiles = tiles_m * tiles_n;
  const int kb_total = (g.K + BK - 1) / BK;

  // Split-K when the tile grid leaves SMs idle: the split count that minimises (waves of CTAs) x (K
  // blocks per split + a fixed cost of 8 K blocks per CTA for its prologue and partial tile), with at
  // least 4 K blocks per split and the fewest splits on a tie (one CTA per SM: a split count that
  // spills a few CTAs into a second wave doubles the time).
  int splits = 1;
  if (tiles < nsm && s.partial) {
    constexpr int64_t kCtaCost = 8;
    const int64_t per = static_cast<int64_t>(tiles) * BM * BN;
    const int64_t fit = per > 0 ? s.partial_floats / per : 0;
    const int smax = static_cast<int>(std::min<int64_t>(kb_total / 4, fit));
    int64_t best = kb_total + kCtaCost;  // one split, one wave
    for (int c = 2; c <= smax; ++c) {
      const int64_t waves = (static_cast<int64_t>(tiles) * c + nsm - 1) / nsm;
      const int64_t cost = waves * ((kb_total + c - 1) / c + kCtaCost);
      if (cost < best) {
        best = cost;
        splits = c;
      }
    }
  }
  int kb_per_split = (kb_total + splits - 1) / splits;
  splits = (kb_total + kb_per_split - 1) / kb_per_split;

  GemmArgs a{};
  a.M = g.M;
  a.N = g.N;
  a.K = g.K;
  a.kb_total = kb_total;
  a.kb_per_split = kb_per_split;
  a.splits = splits;
  a.tiles_m = tiles_m;
  a.tiles_n = tiles_n;
  a.alpha = g.alpha;
  a.beta = g.beta;
  a.C = g.out.C;
  a.ldc = g.out.ldc;
  a.D = g.out.D;
  a.ldd = g.out.ldd;
  a.Dh = g.out.Dh;
  a.Dl = g.out.Dl;
  a.ldh = g.out.ldh;
  a.out_mode = g.out_prec == LATER_PREC_BF16 ? 1 : (g.out_prec == LATER_PREC_SPLIT3 ? 2 : 0);  // SPLIT2: hi only
  a.lower = g.out.lower;
  a.diag = g.out.diag;
  a.shadow_acc = g.out.shadow_acc;
  a.round_prod = g.out.round_prod;
  a.ab_bf16 = bf16 ? 1 : 0;
  a.partial = s.partial;
  a.counters = s.counters;
  a.status = device_status_ptr();
  a.budget = budget > 0 ? budget : kDefaultBudgetCycles;

  // Tensor maps over the stored (column-major) operands.
  CUtensorMap ma{}, mb{}, mal{}, mbl{};
  const uint64_t a_rows = a_mn ? g.M : g.K, a_cols = a_mn ? g.K : g.M;
  const uint64_t b_rows = b_mn ? g.N : g.K, b_cols = b_mn ? g.K : g.N;
  const uint32_t a_box_c = a_mn ? BK : BM;
  const uint32_t b_box_c = b_mn ? BK : BN;
  if (!make_map16(&ma, g.A.hi, a_rows, a_cols, g.A.ld, 64, a_box_c, bf16)) return LATER_ERR_INVALID_ARG;
  if (!make_map16(&mb, g.B.hi, b_rows, b_cols, g.B.ld, 64, b_box_c, bf16)) return LATER_ERR_INVALID_ARG;
  mal = ma;
  mbl = mb;
  if (split3 || split_a) {
    if (!make_map16(&mal, g.A.lo, a_rows, a_cols, g.A.ld, 64, a_box_c, false)) return LATER_ERR_INVALID_ARG;
  }
  if (split3) {
    if (!make_map16(&mbl, g.B.lo, b_rows, b_cols, g.B.ld, 64, b_box_c, false)) return LATER_ERR_INVALID_ARG;
  }

  dim3 grid(tiles, splits);
  TraceScope trace(st, TRACE_GEMM, 2.0 * g.M * g.N * static_cast<double>(g.K));
  if (splits == 1 && !b_mn && persistent_enabled()) {
    const int ctas = tiles < nsm ? tiles : nsm;
    later_status_t r = LATER_ERR_NOT_SUPPORTED;
    if (split3) {
      if (BN == 128) r = launch_persistent_ab<128, 2, 3, 2>(a_mn, b_mn, ma, mb, mal, mbl, a, ctas, st);
    } else if (split_a) {
      if (BN == 256) r = launch_persistent_ab<256, 1, 3, 1>(a_mn, b_mn, ma, mb, mal, mbl, a, ctas, st);
      else if (BN == 128) r = launch_persistent_ab<128, 1, 4, 2>(a_mn, b_mn, ma, mb, mal, mbl, a, ctas, st);
    } else {
      if (BN == 256) r = launch_persistent_ab<256, 0, 4, 2>(a_mn, b_mn, ma, mb, mal, mbl, a, ctas, st);
      else if (BN == 128) r = launch_persistent_ab<128, 0, 6, 2>(a_mn, b_mn, ma, mb, mal, mbl, a, ctas, st);
    }
    if (r != LATER_ERR_NOT_SUPPORTED) return r;
  }
  if (split3) {
    if (BN == 64) return launch_bn<64, 2, 3>(a_mn, b_mn, ma, mb, mal, mbl, a, grid, st);
    return launch_bn<128, 2, 3>(a_mn, b_mn, ma, mb, mal, mbl, a, grid, st);
  }
  if (split_a) {  // A MN-major, B K-major (checked above)
    if (BN == 64) return launch_cfg<64, true, false, 1, 4>(ma, mb, mal, mbl, a, grid, st);
    if (BN == 128) return launch_cfg<128, true, false, 1, 4>(ma, mb, mal, mbl, a, grid, st);
    return launch_cfg<256, true, false, 1, 3>(ma, mb, mal, mbl, a, grid, st);
  }
  if (BN == 64) return launch_bn<64, 0, 6>(a_mn, b_mn, ma, mb, mal, mbl, a, grid, st);
  if (BN == 128) return launch_bn<128, 0, 4>(a_mn, b_mn, ma, mb, mal, mbl, a, grid, st);
  return launch_bn<256, 0, 4>(a_mn, b_mn, ma, mb, mal, mbl, a, grid, st);
}

}  // namespace later
