// Block sub-projection of obstacle-free blocks on the 5th-generation tensor
// cores: Y = X M^T (X: blocks x faces, M: interior rows x faces, the dense
// matrix of ZQ_InitSubMatPoisson3D, Utils3D:1151-1391) with tcgen05.mma in TF32
// and the 3xTF32 split for FP32 accuracy:
//   xh = x rounded to TF32 (10 mantissa bits, nearest even), xl = x - xh
//   (exact) rounded to TF32, so the hardware's TF32 reads change neither;
//   x m ~ xh mh + xh ml + xl mh   (the xl ml term, <= 2^-22 |x m|, is dropped).
// One CTA of 128 threads owns a tile of 128 blocks x BN rows; the sums live in
// tensor memory (128 lanes x BN fp32 columns) as two accumulators, the main
// products xh mh in one and the small corrections xh ml + xl mh in the other,
// added in FP32 at the end: the tensor cores' accumulation rounding then acts
// on one third of the accumulation steps of the large sum.
//
// Operands are stored in global memory as the exact shared-memory images the
// MMAs read: per (tile, chunk of 16 faces) the hi then the lo tile, each row
// 64 bytes in the 64-byte-swizzled K-major layout.  So one chunk is two
// contiguous bulk copies (cp.async.bulk, 16 KB of X and 2 BN x 64 bytes of M)
// whose arrival an mbarrier counts in bytes.  Warp 0 (one lane) produces:
// waits for a stage to be released, posts the byte count, issues the copies;
// warp 1 (one lane) consumes: waits for the bytes, issues the 6 MMAs of the
// chunk (3 products x 2 K-steps of 8) and commits them to the stage's release
// barrier; a last commit marks the accumulators complete.  Then all four warps
// read the accumulators with tcgen05.ld (one TMEM lane per thread = one block)
// and write each interior face through a per-row offset table.
//
// Every wait is bounded: on timeout the CTA records an error flag, stops
// issuing work, waits (bounded) for what it issued, frees its tensor memory
// and returns; the host reports the flag.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "zqs_coarse.h"

namespace zqs {

namespace {

constexpr int kTcM = 128;         // blocks per tile (MMA M)
constexpr int kTcK = 16;          // faces per K chunk (64 bytes of fp32)
constexpr int kTcPad = 32;        // faces are padded to a multiple of this
constexpr int kTcThreads = 128;   // one TMEM lane per thread
constexpr int kTcMaxStages = 8;
constexpr int kTcMaxN = 256;      // rows per tile at most (MMA N)
constexpr uint32_t kTcTmemCols = 512;   // two accumulators of up to 256 columns
constexpr uint32_t kTcCorr = 256;       // column of the correction accumulator
constexpr int kTileA = kTcM * kTcK * 4;      // 8 KB: one hi or lo tile of X
constexpr int kSmemBudget = 224 * 1024;       // dynamic: 227 KB less the kernel's static shared memory
constexpr int kSmemExtra = 1024 + 256;       // alignment slack, barriers, TMEM address
constexpr long long kWaitLimit = 1LL << 24;  // try_wait polls before a wait gives up
constexpr long long kInjectWaitLimit = 1LL << 12;  // the same with the stall injected (test hook)

// FP32 -> TF32 (1 + 8 + 10 bits) by round to nearest even, as an FP32 bit pattern.
__host__ __device__ __forceinline__ uint32_t tf32_rne_bits(uint32_t b) {
    return (b + 0x0FFFu + ((b >> 13) & 1u)) & 0xFFFFE000u;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for the completion of the phase with this parity.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long long limit) {
    for (long long n = 0; n < limit; n++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// Contiguous global -> shared copy whose bytes the mbarrier counts.
__device__ __forceinline__ void bulk_copy(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

// Byte offset of element (row r, face f of the chunk) in a 64-byte-swizzled
// K-major tile image: 16-byte chunk c = f / 4 of row r sits at c ^ ((r >> 1) & 3).
__host__ __device__ __forceinline__ uint32_t sw64_offset(int r, int f) {
    return (uint32_t)(r * 64 + ((((f >> 2) ^ ((r >> 1) & 3)) & 3) << 4) + (f & 3) * 4);
}

// Shared-memory matrix descriptor: K-major operand, 64-byte swizzle (16-byte
// chunk c of row r stored at chunk c ^ ((r >> 1) & 3)), rows 64 bytes apart,
// 8-row groups 512 bytes apart.
__device__ __forceinline__ uint64_t sw64_desc(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;             // leading byte offset (unused by this layout)
    d |= (uint64_t)(512 >> 4) << 32;    // stride byte offset
    d |= (uint64_t)1 << 46;             // descriptor version
    d |= (uint64_t)4 << 61;             // 64-byte swizzle
    return d;
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(da), "l"(db), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

// 16 consecutive fp32 columns of this warp's 32 TMEM lanes (one per thread).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
        "%14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}

__global__ void __launch_bounds__(kTcThreads, 1)
    k_subproj_tc(Layout L, Layout Lc, int s, int rows, int nblocks, int nk, int bn,
                 const unsigned char* __restrict__ Xs, const unsigned char* __restrict__ Ms,
                 const uint8_t* __restrict__ bobs, float* __restrict__ u, float* __restrict__ v,
                 float* __restrict__ w, int nstages, int* __restrict__ err, long long wait_limit, int stall) {
    extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
    // 1024-byte alignment for the swizzle atoms
    const uint32_t raw = smem_u32(tc_smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    unsigned char* gbase = tc_smem_raw + (base - raw);
    const int tile_b = bn * kTcK * 4;                     // a multiple of 1024 (bn % 16 == 0)
    const int bytes_a = 2 * kTileA, bytes_b = 2 * tile_b;  // hi + lo images, contiguous
    const int stage_bytes = bytes_a + bytes_b;
    const uint32_t full = base + nstages * stage_bytes;   // nstages "bytes landed" barriers
    const uint32_t empty = full + 8 * kTcMaxStages;       // nstages "stage released" barriers
    const uint32_t done = empty + 8 * kTcMaxStages;       // accumulators complete
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(gbase + nstages * stage_bytes + 16 * kTcMaxStages + 16);
    __shared__ int s_fail;
    // per row of the tile: the face's offset from its block's corner cell in
    // the padded layout (i + j px + k plane) and its component, -1 past the rows
    __shared__ int s_off[kTcMaxN];
    __shared__ int s_comp[kTcMaxN];

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n0 = blockIdx.x * bn;        // first row of the tile
    const int b0 = blockIdx.y * kTcM;      // first block of the tile

    for (int q = tid; q < bn; q += kTcThreads) {
        const int row = n0 + q;
        int comp = -1, off = 0;
        if (row < rows) off = subproj_block_face(L, s, subproj_interior_face(s, row), 0, 0, 0, comp) - lidx(L, 0, 0, 0);
        s_off[q] = off;
        s_comp[q] = comp;
    }
    if (tid == 0) {
        s_fail = 0;
        for (int q = 0; q < nstages; q++) {
            mbar_init(full + 8 * q, 1);
            mbar_init(empty + 8 * q, 1);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(kTcTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    const unsigned char* xs = Xs + (size_t)blockIdx.y * nk * bytes_a;
    const unsigned char* ms = Ms + (size_t)blockIdx.x * nk * bytes_b;
    int produced = 0;  // producer: chunks whose copies were issued
    if (warp == 0 && lane == 0) {
        // stall (test hook): issue nothing, so the MMA lane's first wait runs
        // out with no copy and no MMA in flight
        for (int j = 0; j < (stall ? 0 : nk); j++) {
            const int st = j % nstages;
            // the stage's previous chunk (j - nstages) released by its MMAs
            if (j >= nstages && !mbar_wait(empty + 8 * st, (uint32_t)((j / nstages - 1) & 1), wait_limit)) {
                s_fail = 1;
                break;
            }
            if (s_fail) break;
            const uint32_t sa = base + st * stage_bytes;
            mbar_expect_tx(full + 8 * st, (uint32_t)stage_bytes);
            bulk_copy(sa, xs + (size_t)j * bytes_a, (uint32_t)bytes_a, full + 8 * st);
            bulk_copy(sa + bytes_a, ms + (size_t)j * bytes_b, (uint32_t)bytes_b, full + 8 * st);
            produced = j + 1;
        }
    } else if (warp == 1 && lane == 0) {
        // kind::tf32: D f32 (bits 4-5 = 1), A and B tf32 (bits 7-9, 10-12 = 2),
        // both K-major, N >> 3 at bit 17, M >> 4 at bit 24
        const uint32_t idesc =
            (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(bn >> 3) << 17) | ((uint32_t)(kTcM >> 4) << 24);
        int consumed = 0;
        for (int kc = 0; kc < nk; kc++) {
            const int st = kc % nstages;
            if (!mbar_wait(full + 8 * st, (uint32_t)((kc / nstages) & 1), wait_limit)) {
                s_fail = 1;
                break;
            }
            if (s_fail) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa = base + st * stage_bytes;
            const uint32_t ah = sa, al = sa + kTileA, bh = sa + bytes_a, bl = sa + bytes_a + tile_b;
#pragma unroll
            for (int k = 0; k < kTcK / 8; k++) {
                const uint32_t off = k * 32;  // 8 tf32 = 32 bytes along K
                const uint32_t acc = (kc > 0 || k > 0) ? 1u : 0u;
                mma_tf32(tmem, sw64_desc(ah + off), sw64_desc(bh + off), idesc, acc);
                mma_tf32(tmem + kTcCorr, sw64_desc(ah + off), sw64_desc(bl + off), idesc, acc);
                mma_tf32(tmem + kTcCorr, sw64_desc(al + off), sw64_desc(bh + off), idesc, 1u);
            }
            mma_commit(empty + 8 * st);
            consumed = kc + 1;
        }
        // the accumulators are complete when every MMA issued so far is
        if (consumed > 0) mma_commit(done);
        if (consumed < nk) s_fail = 1;
    }
    __syncthreads();
    const bool ok = !s_fail;
    // bounded waits for everything issued, whatever happened
    if (tid == 0 && !mbar_wait(done, 0u, wait_limit)) s_fail = 1;
    if (warp == 0 && lane == 0 && !ok) {
        // copies issued but never consumed still land before the CTA leaves
        for (int j = (produced > nstages ? produced - nstages : 0); j < produced; j++)
            mbar_wait(full + 8 * (j % nstages), (uint32_t)((j / nstages) & 1), wait_limit);
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!s_fail) {
        const int gb = b0 + tid;  // this thread's block (TMEM lane tid)
        const bool live = gb < nblocks && !bobs[gb];
        const int bi = gb % Lc.W, bj = (gb / Lc.W) % Lc.H, bk = gb / (Lc.W * Lc.H);
        const int corner = lidx(L, bi * s, bj * s, bk * s);
        const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
        for (int c0 = 0; c0 < bn; c0 += 16) {
            uint32_t r[16], rc[16];
            tmem_ld16(lane_base + (uint32_t)c0, r);
            tmem_ld16(lane_base + kTcCorr + (uint32_t)c0, rc);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (live) {
#pragma unroll
                for (int q = 0; q < 16; q++) {
                    const int comp = s_comp[c0 + q];
                    if (comp >= 0)
                        (comp == 0 ? u : (comp == 1 ? v : w))[corner + s_off[c0 + q]] =
                            __uint_as_float(r[q]) + __uint_as_float(rc[q]);
                }
            }
        }
    } else if (tid == 0) {
        atomicExch(err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcTmemCols)
                     : "memory");
    }
}

// The xh / xl pair of one value at (tile t, row r, face q) of the images.
__device__ __forceinline__ void store_split(unsigned char* __restrict__ Xs, int nk, int t, int r, int q, float x) {
    const float hi = __uint_as_float(tf32_rne_bits(__float_as_uint(x)));
    const float lo = __uint_as_float(tf32_rne_bits(__float_as_uint(x - hi)));
    unsigned char* img = Xs + ((size_t)t * nk + q / kTcK) * (2 * kTileA);
    const uint32_t o = sw64_offset(r, q % kTcK);
    *reinterpret_cast<float*>(img + o) = hi;
    *reinterpret_cast<float*>(img + kTileA + o) = lo;
}

// Block faces gathered and split into the swizzled tile images: per (128-block
// tile t, chunk c of 16 faces) the 8 KB hi image then the lo one; faces past nf
// and blocks past nblocks are 0.  One CTA per block; face q's position in the
// block comes from ftab[q] = i | j << 8 | k << 16 | component << 24.
__global__ void __launch_bounds__(256) k_gather_split_tf32(Layout L, Layout Lc, int s, int nf, int nblocks, int nk,
                                                           const uint32_t* __restrict__ ftab,
                                                           const float* __restrict__ u, const float* __restrict__ v,
                                                           const float* __restrict__ w,
                                                           unsigned char* __restrict__ Xs) {
    const int b = blockIdx.x;
    const int kpad = nk * kTcK;
    const bool live = b < nblocks;
    const int bi = b % Lc.W, bj = (b / Lc.W) % Lc.H, bk = b / (Lc.W * Lc.H);
    const int corner = live ? lidx(L, bi * s, bj * s, bk * s) : 0;
    const int t = b / kTcM, r = b % kTcM;
    for (int q = threadIdx.x; q < kpad; q += blockDim.x) {
        float x = 0.0f;
        if (live && q < nf) {
            const uint32_t f = __ldg(ftab + q);
            const int off = (int)(f & 255u) + (int)((f >> 8) & 255u) * L.px + (int)((f >> 16) & 255u) * (int)L.plane;
            const uint32_t comp = f >> 24;
            x = __ldg((comp == 0 ? u : (comp == 1 ? v : w)) + corner + off);
        }
        store_split(Xs, nk, t, r, q, x);
    }
}


struct MSplit {
    unsigned char* img = nullptr;  // per (row tile, chunk): hi image then lo image, bn x 64 bytes each
    uint32_t* ftab = nullptr;      // per block face: i | j << 8 | k << 16 | component << 24
    int kpad = 0, bn = 0, ntiles = 0;
};
std::mutex g_ms_mu;
std::map<int, MSplit> g_ms;

int get_msplit(int s, MSplit& out) {
    std::lock_guard<std::mutex> lk(g_ms_mu);
    auto it = g_ms.find(s);
    if (it != g_ms.end()) {
        out = it->second;
        return ZQS_OK;
    }
    const std::vector<float> M = coarse_submatrix(s);
    const int nf = 3 * s * s * (s + 1), rows = 3 * s * s * (s - 1);
    MSplit m;
    m.kpad = (nf + kTcPad - 1) / kTcPad * kTcPad;
    m.ntiles = (rows + kTcMaxN - 1) / kTcMaxN;
    m.bn = ((rows + m.ntiles - 1) / m.ntiles + 15) / 16 * 16;
    const int nk = m.kpad / kTcK;
    const size_t tile = (size_t)m.bn * kTcK * 4;
    const size_t bytes = (size_t)m.ntiles * nk * 2 * tile;
    std::vector<unsigned char> img(bytes, 0);
    for (int row = 0; row < rows; row++)
        for (int q = 0; q < nf; q++) {
            const float x = M[(size_t)row * nf + q];
            uint32_t bits;
            std::memcpy(&bits, &x, 4);
            bits = tf32_rne_bits(bits);
            float hi, lo;
            std::memcpy(&hi, &bits, 4);
            const float rest = x - hi;
            std::memcpy(&bits, &rest, 4);
            bits = tf32_rne_bits(bits);
            std::memcpy(&lo, &bits, 4);
            const int t = row / m.bn, r = row % m.bn, c = q / kTcK, f = q % kTcK;
            unsigned char* im = img.data() + ((size_t)t * nk + c) * 2 * tile;
            const uint32_t o = sw64_offset(r, f);
            std::memcpy(im + o, &hi, 4);
            std::memcpy(im + tile + o, &lo, 4);
        }
    // face table: the padded index in a layout with 256-wide rows and 256-row
    // planes is exactly i + 256 j + 65536 k
    std::vector<uint32_t> ft(nf);
    Layout P{};
    P.px = 256;
    P.py = 256;
    for (int q = 0; q < nf; q++) {
        int comp;
        const int packed = subproj_block_face(P, s, q, 0, 0, 0, comp);
        ft[q] = (uint32_t)packed | ((uint32_t)comp << 24);
    }
    ZQS_CUDA_TRY(dev_alloc(&m.img, bytes));
    cudaError_t e = dev_alloc(&m.ftab, ft.size() * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemcpy(m.img, img.data(), bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(m.ftab, ft.data(), ft.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(m.img);
        cudaFree(m.ftab);
        return cuda_fail(e, "tensor-core sub-projection matrix upload");
    }
    g_ms[s] = m;
    out = m;
    return ZQS_OK;
}

}  // namespace

int subproj_tc_prepare(int s) {
    MSplit m;
    int rc = get_msplit(s, m);
    if (rc) return rc;
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [] {
        attr = cudaFuncSetAttribute(k_subproj_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBudget);
    });
    ZQS_CUDA_TRY(attr);
    return ZQS_OK;
}

size_t subproj_tc_split_bytes(int nblocks, int nf) {
    const long long kpad = (nf + kTcPad - 1) / kTcPad * kTcPad;
    const long long bpad = (nblocks + kTcM - 1) / kTcM * kTcM;
    return (size_t)(2 * bpad * kpad) * sizeof(float);
}

std::atomic<int> g_tc_stall{0};

int launch_subproj_tc(const Layout& L, const Layout& Lc, int s, int nf, int rows, int nblocks, float* Xsplit,
                      const uint8_t* bobs, float* u, float* v, float* w, int* err, cudaStream_t st,
                      LaunchCounter& lc) {
    MSplit m;
    {
        // prepared by subproj_tc_prepare (no allocation here: this may run
        // inside a stream capture)
        std::lock_guard<std::mutex> lk(g_ms_mu);
        auto it = g_ms.find(s);
        if (it == g_ms.end()) {
            set_error("tensor-core sub-projection: matrix for this sub_size not prepared");
            return ZQS_ENOTREADY;
        }
        m = it->second;
    }
    // as many stages as fit (2 .. kTcMaxStages)
    const int stage_bytes = 2 * kTileA + 2 * m.bn * kTcK * 4;
    const int nstages = std::min(kTcMaxStages, (kSmemBudget - kSmemExtra) / stage_bytes);
    if (nstages < 2) {
        set_error("tensor-core sub-projection: the operand stages do not fit in shared memory");
        return ZQS_EUNSUPPORTED;
    }
    const size_t smem = (size_t)nstages * stage_bytes + kSmemExtra;
    const int nk = m.kpad / kTcK;
    const long long bpad = (nblocks + kTcM - 1) / kTcM * kTcM;
    unsigned char* Xs = reinterpret_cast<unsigned char*>(Xsplit);
    k_gather_split_tf32<<<(unsigned)bpad, 256, 0, st>>>(L, Lc, s, nf, nblocks, nk, m.ftab, u, v, w, Xs);
    const dim3 grid(m.ntiles, (unsigned)(bpad / kTcM), 1);
    const int stall = g_tc_stall.load(std::memory_order_relaxed);
    k_subproj_tc<<<grid, kTcThreads, smem, st>>>(L, Lc, s, rows, nblocks, nk, m.bn, Xs, m.img, bobs, u, v, w,
                                                 nstages, err, stall ? kInjectWaitLimit : kWaitLimit, stall);
    lc.n += 2;
    ZQS_LAUNCH_CHECK("k_subproj_tc");
    return ZQS_OK;
}

}  // namespace zqs

extern "C" ZQS_API int zqs_debug_inject_tc_stall(int enable) {
    zqs::g_tc_stall.store(enable ? 1 : 0, std::memory_order_relaxed);
    return ZQS_OK;
}
