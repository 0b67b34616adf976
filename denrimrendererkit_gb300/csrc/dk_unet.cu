// Kernels of the learned denoiser (dk_unet_* in include/denrim_cuda.h): a
// 5-level U-Net over the tracer's beauty + albedo + normal + depth AOVs.
//
// Tensors are NHWC bf16 with channel counts that are multiples of 16; a
// tensor may be a channel slice of a wider buffer (leading dimension `ld`,
// channel offset), so the decoder's concat(upsampled, skip) inputs are written
// in place.  3x3 convolutions (stride 1, zero padding 1) are implicit GEMMs
// on the tensor cores with FP32 accumulation:
//   forward   out[p][co] = act(b[co] + sum_{tap, ci} in[p + tap][ci] w[co][tap][ci])
//             M = pixels, N = Cout, K = 9 Cin; also the input gradient, as a
//             forward convolution of the output gradient with the
//             tap-flipped, transposed weights;
//   wgrad     dW[co][tap][ci] += sum_p dOut[p][co] in[p + tap][ci]
//             M = Cout, N = Cin, K = pixels, split over pixel chunks.
// Shared-memory tiles are filled with cp.async (zero fill for the padding)
// through an XOR swizzle that keeps ldmatrix conflict-free.
#include <cstdint>
#include <cstdlib>
#include <initializer_list>

#include <cuda.h>
#include <cuda_bf16.h>

#include "dk_host.h"

namespace dk {
namespace {

__device__ __forceinline__ uint32_t smemAddr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Programmatic dependent launch: the forward pass's kernels are launched so
// that each may start (and set up shared memory, barriers and tensor memory)
// while the previous one drains.  pdlWait() blocks until the previous kernel
// in the stream has completed and its writes are visible; every thread calls
// it before its first global memory access.  pdlRelease() lets the next
// kernel be scheduled.  Both are no-ops for a kernel launched without the
// attribute.
__device__ __forceinline__ void pdlWait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdlRelease() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

// 16-byte async copy; `bytes` 0 fills the destination with zeros.
__device__ __forceinline__ void cpAsync16(void* dst, const void* src, uint32_t bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smemAddr(dst)), "l"(src), "r"(bytes));
}
__device__ __forceinline__ void cpAsyncCommit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cpAsyncWait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

__device__ __forceinline__ void ldmatrixX4(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(smemAddr(p)));
}
__device__ __forceinline__ void ldmatrixX4T(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(smemAddr(p)));
}

// D = A (16x16 bf16, row) * B (16x8 bf16, col) + D (fp32).
__device__ __forceinline__ void mmaBf16(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// ------------------------------------------------------------ forward ----
struct ConvArgs {
    const __nv_bfloat16* in;
    const __nv_bfloat16* w;  // [cout][9][cin]
    const float* bias;       // [cout] or null
    __nv_bfloat16* out;
    uint32_t n, h, w_, cin, ldi, cout, ldo, coOff;
    uint32_t M;  // n * h * w
    int act;     // 0 identity, 1 ReLU
    int accumulate;
};

constexpr int kBM = 128;  // pixels per block
constexpr int kBK = 32;   // channels per k step (4 chunks of 16 bytes)
constexpr int kStages = 3;

// Byte offset of 16-byte chunk `seg` (0..3) of row `r` in a 64-byte-row tile.
__device__ __forceinline__ uint32_t swz64(uint32_t r, uint32_t seg) { return r * 64u + ((seg ^ ((r >> 1) & 3u)) << 4); }

template <int BN>
__global__ void __launch_bounds__(128) k_conv3x3_fwd(ConvArgs a) {
    __shared__ __align__(128) unsigned char sA[kStages][kBM * 64];
    __shared__ __align__(128) unsigned char sB[kStages][BN * 64];
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
    const uint32_t HW = a.h * a.w_;
    // This thread loads A row `tid` (one output pixel).
    const uint32_t m = m0 + tid;
    const bool rowValid = m < a.M;
    const uint32_t img = rowValid ? m / HW : 0u, rem = rowValid ? m - img * HW : 0u;
    const int py = (int)(rem / a.w_), px = (int)(rem - (rem / a.w_) * a.w_);
    const uint32_t chunks = (a.cin + kBK - 1) / kBK;
    const uint32_t kIters = 9u * chunks;

    auto loadStage = [&](uint32_t it, int stage) {
        uint32_t tap = it / chunks, c0 = (it - tap * chunks) * kBK;
        int dy = (int)(tap / 3u) - 1, dx = (int)(tap % 3u) - 1;
        int yy = py + dy, xx = px + dx;
        bool inb = rowValid && yy >= 0 && yy < (int)a.h && xx >= 0 && xx < (int)a.w_;
        const __nv_bfloat16* src =
            inb ? a.in + ((size_t)(img * a.h + (uint32_t)yy) * a.w_ + (uint32_t)xx) * a.ldi + c0 : a.in;
#pragma unroll
        for (uint32_t seg = 0; seg < 4; ++seg) {
            bool v = inb && c0 + seg * 8u < a.cin;
            cpAsync16(&sA[stage][swz64(tid, seg)], v ? src + seg * 8u : a.in, v ? 16u : 0u);
        }
#pragma unroll
        for (uint32_t i = tid; i < (uint32_t)BN * 4u; i += 128u) {
            uint32_t row = i >> 2, seg = i & 3u;
            bool v = c0 + seg * 8u < a.cin;
            const __nv_bfloat16* wsrc = a.w + ((size_t)(n0 + row) * 9u + tap) * a.cin + c0 + seg * 8u;
            cpAsync16(&sB[stage][swz64(row, seg)], v ? wsrc : a.w, v ? 16u : 0u);
        }
    };

    float acc[2][BN / 8][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < BN / 8; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.0f;

#pragma unroll
    for (int s = 0; s < kStages - 1; ++s) {
        if ((uint32_t)s < kIters) loadStage(s, s);
        cpAsyncCommit();
    }
    for (uint32_t it = 0; it < kIters; ++it) {
        cpAsyncWait<kStages - 2>();
        __syncthreads();
        uint32_t nxt = it + kStages - 1;
        if (nxt < kIters) loadStage(nxt, (int)(nxt % kStages));
        cpAsyncCommit();
        const int st = (int)(it % kStages);
#pragma unroll
        for (uint32_t kk = 0; kk < 2; ++kk) {
            uint32_t af[2][4];
#pragma unroll
            for (uint32_t mt = 0; mt < 2; ++mt) {
                uint32_t r = warp * 32u + mt * 16u + (lane & 15u);
                uint32_t seg = kk * 2u + (lane >> 4);
                ldmatrixX4(af[mt][0], af[mt][1], af[mt][2], af[mt][3], &sA[st][swz64(r, seg)]);
            }
#pragma unroll
            for (uint32_t np = 0; np < (uint32_t)BN / 16u; ++np) {
                uint32_t r = np * 16u + (lane & 7u) + ((lane >> 4) << 3);
                uint32_t seg = kk * 2u + ((lane >> 3) & 1u);
                uint32_t b0, b1, b2, b3;
                ldmatrixX4(b0, b1, b2, b3, &sB[st][swz64(r, seg)]);
#pragma unroll
                for (uint32_t mt = 0; mt < 2; ++mt) {
                    mmaBf16(acc[mt][2 * np], af[mt], b0, b1);
                    mmaBf16(acc[mt][2 * np + 1], af[mt], b2, b3);
                }
            }
        }
    }
    cpAsyncWait<0>();
    // Epilogue: bias, activation, optional accumulate, bf16 store.
#pragma unroll
    for (uint32_t mt = 0; mt < 2; ++mt) {
#pragma unroll
        for (uint32_t half = 0; half < 2; ++half) {
            uint32_t row = m0 + warp * 32u + mt * 16u + (lane >> 2) + half * 8u;
            if (row >= a.M) continue;
            __nv_bfloat16* orow = a.out + (size_t)row * a.ldo + a.coOff;
#pragma unroll
            for (uint32_t nt = 0; nt < (uint32_t)BN / 8u; ++nt) {
                uint32_t col = n0 + nt * 8u + (lane & 3u) * 2u;
                float v0 = acc[mt][nt][half * 2 + 0], v1 = acc[mt][nt][half * 2 + 1];
                if (a.bias) {
                    v0 += a.bias[col];
                    v1 += a.bias[col + 1];
                }
                if (a.act == 1) {
                    v0 = fmaxf(v0, 0.0f);
                    v1 = fmaxf(v1, 0.0f);
                }
                __nv_bfloat162* dst = reinterpret_cast<__nv_bfloat162*>(orow + col);
                if (a.accumulate) {
                    float2 o = __bfloat1622float2(*dst);
                    v0 += o.x;
                    v1 += o.y;
                }
                *dst = __floats2bfloat162_rn(v0, v1);
            }
        }
    }
}

// ------------------------------------------------- tcgen05 forward ----
// The same convolution on the 5th-generation tensor cores: one CTA computes
// 128 output pixels x all Cout (one tcgen05.mma of M = 128, N = Cout, K = 16
// per 16 input channels of a tap), accumulating in tensor memory.  Operand
// tiles are K-major with the 128-byte swizzle: 64 channels (128 bytes) per
// row, 8-row atoms of 1024 bytes; cp.async fills them (zero fill for the
// padding), one thread issues the MMAs and commits each stage to an
// mbarrier that the copies of the stage's next use wait on.  Every wait is
// bounded: on timeout the kernel records an error, waits (bounded) for its
// MMAs, frees its tensor memory and returns.
constexpr int kTcStages = 4;
constexpr uint32_t kTcRows = 128;

__device__ int g_unetError;

__device__ __forceinline__ uint64_t umaDesc(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4)  // start address
           | ((uint64_t)1 << 16)                // leading byte offset (unused for swizzled K-major)
           | ((uint64_t)(1024u >> 4) << 32)     // stride byte offset: 8 rows x 128 B
           | ((uint64_t)1 << 46)                // descriptor version
           | ((uint64_t)2 << 61);               // 128-byte swizzle
}

// tcgen05.mma kind::f16 with both shared-memory descriptors given as their
// low words (start address >> 4 in bits 0-13, leading byte offset) and the
// high word they share (stride byte offset, version, 128-byte swizzle): an
// operand's position inside a tile is then one 32-bit add, and the single
// issuing thread spends a few instructions per MMA.
__device__ __forceinline__ uint32_t descLo(uint32_t saddr) { return (uint32_t)umaDesc(saddr); }
__device__ __forceinline__ uint32_t descHi() { return (uint32_t)(umaDesc(0u) >> 32); }
__device__ __forceinline__ void mmaF16(uint32_t d, uint32_t aLo, uint32_t bLo, uint32_t hi, uint32_t idesc,
                                       uint32_t acc) {
    asm volatile(
        "{\n.reg .pred p;\n.reg .b64 da, db;\nsetp.ne.b32 p, %5, 0;\nmov.b64 da, {%1, %3};\nmov.b64 db, {%2, %3};\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], da, db, %4, p;\n}\n" ::"r"(d),
        "r"(aLo), "r"(bLo), "r"(hi), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ bool mbarTryWait(uint32_t bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0u;
}
__device__ __forceinline__ bool mbarWait(uint32_t bar, uint32_t parity) {
    if (mbarTryWait(bar, parity)) return true;
    const long long start = clock64();
    for (;;) {
        if (mbarTryWait(bar, parity)) return true;
        if (clock64() - start > 4000000000ll) return false;  // about 2 s
    }
}

// A slot of an n-slot ring and the parity of its current use, advanced one
// use at a time (no division on the issuing threads' path).
struct RingPos {
    uint32_t slot, phase;
    __device__ __forceinline__ void advance(uint32_t n) {
        if (++slot == n) {
            slot = 0u;
            phase ^= 1u;
        }
    }
};

__global__ void __launch_bounds__(128, 1) k_conv3x3_tc(ConvArgs a, uint32_t tmemCols) {
    extern __shared__ unsigned char dsm[];
    const uint32_t raw = smemAddr(dsm);
    unsigned char* sm = dsm + (((raw + 1023u) & ~1023u) - raw);
    const uint32_t N = a.cout;
    const uint32_t aBytes = kTcRows * 128u, bBytes = N * 128u;
    unsigned char* sA = sm;
    unsigned char* sB = sm + kTcStages * aBytes;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sB + kTcStages * bBytes);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + kTcStages);
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smemAddr(tslot)),
                     "r"(tmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    if (tid == 0) {
        for (int s = 0; s < kTcStages; ++s)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smemAddr(&bars[s])));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t taddr = *tslot;

    const uint32_t m0 = blockIdx.x * kTcRows;
    const uint32_t HW = a.h * a.w_;
    const uint32_t m = m0 + tid;
    const bool rowValid = m < a.M;
    const uint32_t img = rowValid ? m / HW : 0u, rem = rowValid ? m - img * HW : 0u;
    const int py = (int)(rem / a.w_), px = (int)(rem - (rem / a.w_) * a.w_);
    const uint32_t chunks = (a.cin + 63u) / 64u;
    const uint32_t kIters = 9u * chunks;
    // kind::f16 instruction descriptor: D f32, A and B bf16, both K-major, N, M = 128.
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((kTcRows >> 4) << 24);

    auto loadStage = [&](uint32_t it, uint32_t stage) {
        uint32_t tap = it / chunks, c0 = (it - tap * chunks) * 64u;
        int yy = py + (int)(tap / 3u) - 1, xx = px + (int)(tap % 3u) - 1;
        bool inb = rowValid && yy >= 0 && yy < (int)a.h && xx >= 0 && xx < (int)a.w_;
        const __nv_bfloat16* src =
            inb ? a.in + ((size_t)(img * a.h + (uint32_t)yy) * a.w_ + (uint32_t)xx) * a.ldi + c0 : a.in;
        unsigned char* rowA = sA + stage * aBytes + tid * 128u;
#pragma unroll
        for (uint32_t j = 0; j < 8; ++j) {
            bool v = inb && c0 + j * 8u < a.cin;
            cpAsync16(rowA + ((j ^ (tid & 7u)) << 4), v ? src + j * 8u : a.in, v ? 16u : 0u);
        }
        unsigned char* tileB = sB + stage * bBytes;
        for (uint32_t i = tid; i < N * 8u; i += 128u) {
            uint32_t row = i >> 3, j = i & 7u;
            bool v = c0 + j * 8u < a.cin;
            const __nv_bfloat16* wsrc = a.w + ((size_t)row * 9u + tap) * a.cin + c0 + j * 8u;
            cpAsync16(tileB + row * 128u + ((j ^ (row & 7u)) << 4), v ? wsrc : a.w, v ? 16u : 0u);
        }
    };

    bool failed = false;
    uint32_t lastCommitted = 0xffffffffu;
#pragma unroll
    for (int s = 0; s < kTcStages - 1; ++s) {
        if ((uint32_t)s < kIters) loadStage((uint32_t)s, (uint32_t)s);
        cpAsyncCommit();
    }
    for (uint32_t it = 0; it < kIters && !failed; ++it) {
        const uint32_t stage = it % kTcStages;
        cpAsyncWait<kTcStages - 2>();
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t c0 = (it % chunks) * 64u;
            const uint32_t aBase = smemAddr(sA + stage * aBytes), bBase = smemAddr(sB + stage * bBytes);
#pragma unroll
            for (uint32_t ks = 0; ks < 4; ++ks) {
                if (c0 + ks * 16u >= a.cin) break;
                uint64_t ad = umaDesc(aBase + ks * 32u), bd = umaDesc(bBase + ks * 32u);
                uint32_t acc = (it > 0 || ks > 0) ? 1u : 0u;
                asm volatile(
                    "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             smemAddr(&bars[stage]))
                         : "memory");
        }
        lastCommitted = it;
        const uint32_t nxt = it + kTcStages - 1;
        if (nxt < kIters) {
            const uint32_t ps = nxt % kTcStages;
            if (nxt >= (uint32_t)kTcStages) {  // the buffer's previous MMAs (iteration nxt - stages) must be done
                uint32_t use = (nxt - kTcStages) / kTcStages;
                if (!mbarWait(smemAddr(&bars[ps]), use & 1u)) failed = true;
            }
            if (!failed) loadStage(nxt, ps);
        }
        cpAsyncCommit();
    }
    cpAsyncWait<0>();
    bool done = false;
    if (lastCommitted != 0xffffffffu)
        done = mbarWait(smemAddr(&bars[lastCommitted % kTcStages]), (lastCommitted / kTcStages) & 1u);
    if (!done || failed) {
        if (tid == 0) atomicExch(&g_unetError, 1);
    } else {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const uint32_t row = warp * 32u + lane;
        const uint32_t pix = m0 + row;
        __nv_bfloat16* orow = a.out + (size_t)pix * a.ldo + a.coOff;
        for (uint32_t c0 = 0; c0 < N; c0 += 16u) {
            uint32_t r[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                "%14, %15}, [%16];\n"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                : "r"(taddr + ((warp * 32u) << 16) + c0));
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            if (pix >= a.M) continue;
#pragma unroll
            for (uint32_t k = 0; k < 16; k += 2) {
                float v0 = __uint_as_float(r[k]), v1 = __uint_as_float(r[k + 1]);
                uint32_t col = c0 + k;
                if (a.bias) {
                    v0 += a.bias[col];
                    v1 += a.bias[col + 1];
                }
                if (a.act == 1) {
                    v0 = fmaxf(v0, 0.0f);
                    v1 = fmaxf(v1, 0.0f);
                }
                __nv_bfloat162* dst = reinterpret_cast<__nv_bfloat162*>(orow + col);
                if (a.accumulate) {
                    float2 o = __bfloat1622float2(*dst);
                    v0 += o.x;
                    v1 += o.y;
                }
                *dst = __floats2bfloat162_rn(v0, v1);
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(tmemCols));
}

size_t tcSmemBytes(uint32_t cout) { return (size_t)kTcStages * (kTcRows * 128u + cout * 128u) + 1024u + 64u; }

// ------------------------------------------- tcgen05 + TMA, persistent ----
// The production convolution.  Persistent CTAs (one per SM) walk output
// tiles of 128 pixels (th image rows x tw columns, tw a power of two <= 128)
// with three warp roles:
//   warp 0     TMA producer: per (tap, 64-channel chunk) one 4-D box of the
//              activation tensor {64 ch, tw, th, 1} at the tap-shifted
//              coordinate (out-of-range pixels and channels are zero filled
//              by the copy engine) and one 3-D box of the weights
//              {64 ch, 1 tap, Cout}, both into 128-byte-swizzled K-major tiles;
//   warp 1     MMA issuer: tcgen05.mma M = 128, N = Cout, K = 16 into one of
//              the tensor-memory accumulators, stage release and
//              accumulator hand-off through tcgen05.commit;
//   warps 2-9  epilogue: tcgen05.ld of their TMEM lane quarter (two warps
//              per quarter, each half of the channels), bias, ReLU, optional
//              accumulate, bf16 stores; the next tiles' MMAs run into the
//              other accumulators (up to four) meanwhile.
// Every mbarrier wait is bounded (about 2 s); a role that times out records
// the error and stops, the others then time out in turn, and the CTA frees
// its tensor memory before returning.
constexpr uint32_t kHaloPix = 130;          // 128 output pixels and one on each side
constexpr uint32_t kHaloSlotBytes = 17408;  // 130 rows of 128 B, padded to 17 x 1024 B
constexpr uint32_t kTmaStagesMin = 4;   // (tap, chunk) stages in flight: at least 4,
constexpr uint32_t kTmaStagesMax = 8;   // more where shared memory holds them
constexpr uint32_t kTmaBarBytes = 256;  // full[8] empty[8] accFull[4] accEmpty[4], TMEM slot, flag

struct TmaConvArgs {
    const float* bias;
    __nv_bfloat16* out;
    uint32_t n, h, w, cin, cout, ldo, coOff, tw, th, tilesX, tilesY, numTiles, chunks, cols;
    uint32_t stages;  // kTmaStagesMin..kTmaStagesMax
    int act, accumulate;
    int staged;  // epilogue rows through shared memory (see epilogueRow)
};

__device__ __forceinline__ void mbarInit(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbarArrive(uint32_t bar) {
    asm volatile("{\n.reg .b64 st;\nmbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbarExpectTx(uint32_t bar, uint32_t bytes) {
    asm volatile("{\n.reg .b64 st;\nmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}\n" ::"r"(bar),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void tmaLoad4(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                         uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];\n" ::"r"(dst),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
        : "memory");
}
__device__ __forceinline__ void tmaLoad3(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(dst),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
        : "memory");
}
__device__ __forceinline__ void umaCommit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
                 : "memory");
}

// The epilogue: eight warps, two per tensor-memory lane quarter (32 output
// pixels each).  When Cout is a multiple of 32 the two warps of a quarter
// split every accumulator's channels in halves; otherwise the first takes all
// of them and the second has nothing to do.  Up to four accumulators (as many
// as tensor memory holds, at least two) let the MMA warp run ahead of them.
constexpr uint32_t kEpiWarps = 8;
__host__ __device__ constexpr bool epiSplit(uint32_t n) { return n % 32u == 0u; }
__host__ __device__ constexpr uint32_t epiCols(uint32_t n) { return epiSplit(n) ? n / 2u : n; }
// Shared memory one epilogue warp uses to transpose its part of an output
// row: 32 pixels of its channels at a pitch of 2 x channels + 16 bytes (an odd
// number of 16-byte units, so eight lanes' 16-byte writes fall on distinct
// banks), then the 32 pixels' global row pointers.
__host__ __device__ constexpr uint32_t epiPitch(uint32_t cols) { return 2u * cols + 16u; }
__host__ __device__ constexpr uint32_t epiWarpBytes(uint32_t n) { return 32u * epiPitch(epiCols(n)) + 32u * 8u; }
// The same for a warp that takes all N channels of its rows.
__host__ __device__ constexpr uint32_t epiWarpBytesAll(uint32_t n) { return 32u * epiPitch(n) + 32u * 8u; }
__host__ __device__ constexpr uint32_t accBuffers(uint32_t cols) { return 4u * cols <= 512u ? 4u : 2u; }

// This warp's channels [c0, c1) of one accumulator (its 32 TMEM lanes: 32
// output pixels) to global memory: bias, ReLU, bf16, optionally added to the
// destination.  `src` is the accumulator's TMEM address for the warp's lane
// quarter, `dst` this lane's pixel (its channel 0), nullptr outside the image.
// With `stage` the warp writes its part of the row into shared memory and then
// stores every pixel's channels as 16-byte pieces by consecutive lanes, and
// hands the accumulator back as soon as it is read; `stage` is null when the
// destination is accumulated into (its bf16 sum is formed from the FP32
// value, as on the direct path) or not 16-byte aligned.  With `zero` the
// warp clears the columns it read before handing the accumulator back.
__device__ __forceinline__ void zeroColumns(uint32_t src, uint32_t c0, uint32_t c1) {
    const uint32_t z = 0u;
    for (uint32_t c = c0; c < c1; c += 16u)
        asm volatile(
            "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, "
            "%1, %1};\n" ::"r"(src + c),
            "r"(z)
            : "memory");
    asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory");
}

__device__ __forceinline__ void epilogueRow(uint32_t src, uint32_t c0, uint32_t c1, const float* bias, int act,
                                            int accumulate, __nv_bfloat16* dst, unsigned char* stage,
                                            uint32_t accEmptyBar, bool zero = false) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t pitch = epiPitch(c1 - c0);
    const bool biasVec = bias && (reinterpret_cast<uintptr_t>(bias) & 15u) == 0u;
    for (uint32_t c = c0; c < c1; c += 16u) {
        uint32_t rr[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
            "%12, %13, %14, %15}, [%16];\n"
            : "=r"(rr[0]), "=r"(rr[1]), "=r"(rr[2]), "=r"(rr[3]), "=r"(rr[4]), "=r"(rr[5]), "=r"(rr[6]), "=r"(rr[7]),
              "=r"(rr[8]), "=r"(rr[9]), "=r"(rr[10]), "=r"(rr[11]), "=r"(rr[12]), "=r"(rr[13]), "=r"(rr[14]),
              "=r"(rr[15])
            : "r"(src + c));
        float bv[16];
        if (biasVec) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float4 b4 = __ldg(reinterpret_cast<const float4*>(bias + c) + k);
                bv[4 * k] = b4.x;
                bv[4 * k + 1] = b4.y;
                bv[4 * k + 2] = b4.z;
                bv[4 * k + 3] = b4.w;
            }
        } else {
#pragma unroll
            for (int k = 0; k < 16; ++k) bv[k] = bias ? __ldg(bias + c + k) : 0.0f;
        }
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        float v2[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            float x = __uint_as_float(rr[k]);
            if (bias) x += bv[k];
            if (act == 1) x = fmaxf(x, 0.0f);
            v2[k] = x;
        }
        if (stage) {
            uint32_t packed[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                __nv_bfloat162 h2 = __floats2bfloat162_rn(v2[2 * k], v2[2 * k + 1]);
                packed[k] = *reinterpret_cast<uint32_t*>(&h2);
            }
            uint4* sp = reinterpret_cast<uint4*>(stage + lane * pitch + (c - c0) * 2u);
            sp[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
            sp[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
            continue;
        }
        if (!dst) continue;
        __nv_bfloat162* d2 = reinterpret_cast<__nv_bfloat162*>(dst + c);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            float x0v = v2[2 * k], x1v = v2[2 * k + 1];
            if (accumulate) {
                float2 o = __bfloat1622float2(d2[k]);
                x0v += o.x;
                x1v += o.y;
            }
            d2[k] = __floats2bfloat162_rn(x0v, x1v);
        }
    }
    if (zero) zeroColumns(src, c0, c1);  // the next row in this accumulator slot starts from zero
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    mbarArrive(accEmptyBar);
    if (!stage) return;
    __nv_bfloat16** rows = reinterpret_cast<__nv_bfloat16**>(stage + 32u * pitch);
    rows[lane] = dst ? dst + c0 : nullptr;
    __syncwarp();
    // 16-byte pieces: `per` per pixel; lane j takes pieces j, j + 32, ...
    const uint32_t per = (c1 - c0) / 8u;
    const bool pow2 = (per & (per - 1u)) == 0u;
    const uint32_t sh = 31u - __clz(per);
    uint32_t pix = pow2 ? lane >> sh : lane / per;
    uint32_t part = lane - pix * per;
    const uint32_t dq = pow2 ? 32u >> sh : 32u / per, dr = 32u - dq * per;
    for (; pix < 32u; pix += dq) {
        __nv_bfloat16* d = rows[pix];
        if (d) *reinterpret_cast<uint4*>(d + part * 8u) = *reinterpret_cast<const uint4*>(stage + pix * pitch + part * 16u);
        part += dr;
        if (part >= per) {
            part -= per;
            ++pix;
        }
    }
    __syncwarp();
}

// The K steps of one row-tap stage: for dx = 0, 1, 2 the A operand is the
// stage's input row from pixel dx on (128 bytes further per pixel) and the B
// operand the weights of tap (dy, dx); straight-line code (see the halo
// kernel on branches between MMAs).
template <uint32_t kSteps>
__device__ __forceinline__ void rowTapMmas(uint32_t d, uint32_t aLo, uint32_t bLo, uint32_t bTapU, uint32_t hi,
                                           uint32_t idesc, uint32_t acc) {
#pragma unroll
    for (uint32_t dx = 0; dx < 3u; ++dx)
#pragma unroll
        for (uint32_t ks = 0; ks < kSteps; ++ks)
            mmaF16(d, aLo + dx * 8u + 2u * ks, bLo + dx * bTapU + 2u * ks, hi, idesc, (dx | ks) ? 1u : acc);
}

// kRowTap (images at least 128 pixels wide): an output tile is 128 pixels of
// one row and a pipeline stage is (dy, 64-channel chunk): one box of the input
// row y + dy - 1, 130 pixels wide, and the weights of the three taps (dy, 0..2),
// so a tile takes 3 x chunks stages and waits instead of 9 x chunks.
template <bool kRowTap>
__global__ void __launch_bounds__(320, 1)
    k_conv3x3_tma(const __grid_constant__ CUtensorMap mapIn, const __grid_constant__ CUtensorMap mapW, TmaConvArgs a) {
    extern __shared__ unsigned char dsm[];
    const uint32_t raw = smemAddr(dsm);
    unsigned char* sm = dsm + (((raw + 1023u) & ~1023u) - raw);
    const uint32_t N = a.cout;
    const uint32_t aBytes = kRowTap ? kHaloSlotBytes : 128u * 128u, bBytes = (kRowTap ? 3u : 1u) * N * 128u;
    unsigned char* sA = sm;
    const uint32_t S = a.stages;
    unsigned char* sB = sm + S * aBytes;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sB + S * bBytes);
    // bars: full[S], empty[S], accFull[4], accEmpty[4]
    const uint32_t fullBar = smemAddr(bars), emptyBar = fullBar + 8u * kTmaStagesMax;
    const uint32_t accFullBar = emptyBar + 8u * kTmaStagesMax, accEmptyBar = accFullBar + 32u;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2 * kTmaStagesMax + 8);
    const uint32_t nbuf = accBuffers(a.cols), bufShift = nbuf == 4u ? 2u : 1u;
    int* abortFlag = reinterpret_cast<int*>(tslot + 1);
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;

    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smemAddr(tslot)),
                     "r"(nbuf * a.cols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    if (tid == 0) {
        for (uint32_t s = 0; s < S; ++s) {
            mbarInit(fullBar + 8u * s, 1);
            mbarInit(emptyBar + 8u * s, 1);
        }
        for (uint32_t b = 0; b < nbuf; ++b) {
            mbarInit(accFullBar + 8u * b, 1);
            mbarInit(accEmptyBar + 8u * b, epiSplit(N) ? 256u : 128u);
        }
        *abortFlag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(&mapIn) : "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(&mapW) : "memory");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    pdlRelease();
    pdlWait();
    const uint32_t taddr = *tslot;
    const uint32_t txBytes = (kRowTap ? kHaloPix * 128u : aBytes) + bBytes;
    volatile int* abortV = abortFlag;

    if (warp == 0 && kRowTap) {
        if (lane == 0) {
            uint32_t g = 0;
            RingPos pos{0u, 0u};
            bool ok = true;
            for (uint32_t tile = blockIdx.x; ok && tile < a.numTiles && !*abortV; tile += gridDim.x) {
                uint32_t tx = tile % a.tilesX, rest = tile / a.tilesX;
                uint32_t ty = rest % a.tilesY, img = rest / a.tilesY;
                int x0 = (int)(tx * 128u), y0 = (int)ty;
                for (uint32_t dy = 0; ok && dy < 3u; ++dy) {
                    for (uint32_t c = 0; c < a.chunks; ++c, ++g, pos.advance(S)) {
                        if (g >= S && !mbarWait(emptyBar + 8u * pos.slot, pos.phase ^ 1u)) {
                            ok = false;
                            break;
                        }
                        const uint32_t full = fullBar + 8u * pos.slot;
                        mbarExpectTx(full, txBytes);
                        tmaLoad4(smemAddr(sA + pos.slot * aBytes), &mapIn, (int)(c * 64u), x0 - 1, y0 + (int)dy - 1,
                                 (int)img, full);
                        for (uint32_t dx = 0; dx < 3u; ++dx)
                            tmaLoad3(smemAddr(sB + pos.slot * bBytes + dx * N * 128u), &mapW, (int)(c * 64u),
                                     (int)(dy * 3u + dx), 0, full);
                    }
                }
            }
            if (!ok) *abortV = 1;
        }
    } else if (warp == 0) {
        if (lane == 0) {
            uint32_t g = 0;
            RingPos pos{0u, 0u};
            bool ok = true;
            for (uint32_t tile = blockIdx.x; ok && tile < a.numTiles && !*abortV; tile += gridDim.x) {
                uint32_t tx = tile % a.tilesX, rest = tile / a.tilesX;
                uint32_t ty = rest % a.tilesY, img = rest / a.tilesY;
                int x0 = (int)(tx * a.tw), y0 = (int)(ty * a.th);
                for (uint32_t tap = 0; ok && tap < 9u; ++tap) {
                    const int dy = (int)(tap / 3u), dx = (int)tap - 3 * dy;
                    for (uint32_t c = 0; c < a.chunks; ++c, ++g, pos.advance(S)) {
                        if (g >= S && !mbarWait(emptyBar + 8u * pos.slot, pos.phase ^ 1u)) {
                            ok = false;
                            break;
                        }
                        const uint32_t full = fullBar + 8u * pos.slot;
                        mbarExpectTx(full, txBytes);
                        tmaLoad4(smemAddr(sA + pos.slot * aBytes), &mapIn, (int)(c * 64u), x0 + dx - 1, y0 + dy - 1,
                                 (int)img, full);
                        tmaLoad3(smemAddr(sB + pos.slot * bBytes), &mapW, (int)(c * 64u), (int)tap, 0, full);
                    }
                }
            }
            if (!ok) *abortV = 1;
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((128u >> 4) << 24);
            const uint32_t hi = descHi(), aLo0 = descLo(smemAddr(sA)), bLo0 = descLo(smemAddr(sB));
            const uint32_t lastSteps = (a.cin - (a.chunks - 1u) * 64u + 15u) / 16u;
            RingPos pos{0u, 0u};
            uint32_t t = 0;
            for (uint32_t tile = blockIdx.x; tile < a.numTiles && !*abortV; tile += gridDim.x, ++t) {
                uint32_t b = t & (nbuf - 1u), v = t >> bufShift;
                if (v > 0 && !mbarWait(accEmptyBar + 8u * b, (v - 1u) & 1u)) {
                    *abortV = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t dAddr = taddr + b * a.cols;
                bool ok = true;
                uint32_t acc = 0u;
                for (uint32_t it = 0; ok && it < (kRowTap ? 3u : 9u); ++it) {
                    for (uint32_t c = 0; c < a.chunks; ++c, pos.advance(S)) {
                        if (!mbarWait(fullBar + 8u * pos.slot, pos.phase)) {
                            ok = false;
                            break;
                        }
                        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                        // K steps of 16 channels in this (tap, chunk): 4, fewer in a partial last chunk
                        const uint32_t steps = c + 1u < a.chunks ? 4u : lastSteps;
                        const uint32_t aLo = aLo0 + pos.slot * (aBytes >> 4), bLo = bLo0 + pos.slot * (bBytes >> 4);
                        if (kRowTap) {
                            const uint32_t bTapU = (N * 128u) >> 4;
                            if (steps == 4u) rowTapMmas<4>(dAddr, aLo, bLo, bTapU, hi, idesc, acc);
                            else if (steps == 3u) rowTapMmas<3>(dAddr, aLo, bLo, bTapU, hi, idesc, acc);
                            else if (steps == 2u) rowTapMmas<2>(dAddr, aLo, bLo, bTapU, hi, idesc, acc);
                            else rowTapMmas<1>(dAddr, aLo, bLo, bTapU, hi, idesc, acc);
                            acc = 1u;
                            umaCommit(emptyBar + 8u * pos.slot);
                            continue;
                        }
                        mmaF16(dAddr, aLo, bLo, hi, idesc, acc);
                        acc = 1u;
                        if (steps > 1u) mmaF16(dAddr, aLo + 2u, bLo + 2u, hi, idesc, 1u);
                        if (steps > 2u) mmaF16(dAddr, aLo + 4u, bLo + 4u, hi, idesc, 1u);
                        if (steps > 3u) mmaF16(dAddr, aLo + 6u, bLo + 6u, hi, idesc, 1u);
                        umaCommit(emptyBar + 8u * pos.slot);  // the stage is free once these MMAs are done
                    }
                }
                if (!ok) {
                    *abortV = 1;
                    break;
                }
                umaCommit(accFullBar + 8u * b);  // the accumulator is complete
            }
        }
    } else {
        // Epilogue warps 2..9: TMEM lane quarter warp % 4, channel half (warp - 2) / 4.
        const uint32_t q = warp & 3u, half = (warp - 2u) >> 2;
        const uint32_t r = q * 32u + lane;
        const uint32_t cw = epiCols(N), c0 = half * cw, c1 = epiSplit(N) ? c0 + cw : (half ? 0u : N);
        unsigned char* stage =
            a.staged ? reinterpret_cast<unsigned char*>(bars) + kTmaBarBytes + (warp - 2u) * epiWarpBytes(N) : nullptr;
        uint32_t t = 0;
        for (uint32_t tile = blockIdx.x; c1 > c0 && tile < a.numTiles; tile += gridDim.x, ++t) {
            uint32_t b = t & (nbuf - 1u), v = t >> bufShift;
            if (!mbarWait(accFullBar + 8u * b, v & 1u)) {
                *abortV = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            uint32_t tx = tile % a.tilesX, rest = tile / a.tilesX;
            uint32_t ty = rest % a.tilesY, img = rest / a.tilesY;
            uint32_t px = tx * a.tw + r % a.tw, py = ty * a.th + r / a.tw;
            bool valid = px < a.w && py < a.h;
            __nv_bfloat16* orow = valid ? a.out + ((size_t)(img * a.h + py) * a.w + px) * a.ldo + a.coOff : nullptr;
            epilogueRow(taddr + ((q * 32u) << 16) + b * a.cols, c0, c1, a.bias, a.act, a.accumulate, orow, stage,
                        accEmptyBar + 8u * b);
        }
    }
    __syncthreads();
    if (*abortV && tid == 0) atomicExch(&g_unetError, 2);
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(nbuf * a.cols));
}

size_t tmaSmemBytes(uint32_t cout, bool staged, uint32_t stages, bool rowTap) {
    const size_t stage = rowTap ? kHaloSlotBytes + 3u * cout * 128u : 128u * 128u + cout * 128u;
    return (size_t)stages * stage + 1024u + kTmaBarBytes + (staged ? kEpiWarps * epiWarpBytes(cout) : 0u);
}

// -------------------------------------- tcgen05 + TMA, halo-row ring ----
// The convolution for wide, shallow layers (the full- and half-resolution
// levels of the U-Net, where the per-tap kernel above re-reads every input
// pixel nine times from L2 and waits on it).  An output tile is 128
// consecutive pixels of one image row; a persistent CTA walks its share of
// the output rows (an equal, contiguous range of the rows numbered image by
// image, tile column by tile column, top to bottom), down one tile column at
// a time, and keeps the input rows it needs in a ring
// of halo rows: one TMA box {64 channels, 130 pixels} per 64-channel chunk
// and input row, loaded once (zero filled outside the image).  For tap
// (dy, dx) the MMA's A operand is the 128 rows of halo row y - 1 + dy that
// start at pixel dx: a contiguous run of 128-byte rows inside the slot, so all
// nine taps read the same shared-memory rows and each input row crosses L2
// once per tile column.  The weights of the layer (9 x chunks boxes of
// {64 channels, Cout}) stay resident in shared memory for the whole launch.
//   warp 0     TMA producer: the weights once, then the halo rows in order;
//   warp 1     MMA issuer: per output row 9 taps x chunks x K-steps of
//              tcgen05.mma M = 128, N = Cout, K = 16 into one of the TMEM
//              accumulators; releases a halo row once its last reader is done;
//   warps 2-9  epilogue as in k_conv3x3_tma.
// Waits are bounded as there.
constexpr uint32_t kHaloRingMin = 4;        // halo-row slots: three rows in use and one loading at least,
constexpr uint32_t kHaloRingMax = 16;       // and as many more loading as shared memory holds
constexpr uint32_t kHaloBarBytes = 1024;    // full[16] empty[16] weights accFull[32] accEmpty[32], TMEM slot, flag
constexpr uint32_t kHaloAccMax = 32;

struct HaloConvArgs {
    const float* bias;
    __nv_bfloat16* out;
    uint32_t n, h, w, cin, cout, ldo, coOff;
    uint32_t tilesX, totalRows, chunks, cols;  // totalRows = n x tilesX x h output rows of 128 pixels
    uint32_t ring;  // halo-row slots, kHaloRingMin..kHaloRingMax
    uint32_t slots, logSlots;  // stacked variant: accumulator slots of Cout columns (a power of two)
    uint32_t tmaStore;         // stacked variant: output rows leave by TMA tensor stores (Cout 16, 32 or 64)
    int act, accumulate;
    int staged;  // epilogue rows through shared memory (see epilogueRow)
    // With tensor-store rows: the 2x2 average of the output (h, w even) is also
    // written here, [n][h / 2][w / 2][poolLd] (channels 0 .. Cout), or null.
    __nv_bfloat16* pool;
    uint32_t poolLd;
};

// One accumulator slot of the stacked halo kernel to global memory through a
// TMA tensor store: this warp's 32 pixels (TMEM lanes) x all N channels are
// staged as a box {N channels, 32 pixels} in shared memory, laid out with the
// store map's swizzle (16-byte chunk j of pixel row r at r * 2N + 16 (j ^ f(r)),
// f(r) the row's address bits 7.. -- XOR-swizzle over 2N-byte rows, which also
// keeps the eight lanes of a 16-byte store on distinct banks), then one lane
// issues the store of the box at (channel offset, pixel, row, image); pixels
// beyond the image width are clipped by the copy engine.  `buf` alternates
// between two boxes per warp: before writing one, the warp waits until the
// store issued from it two rows earlier has read it.
__device__ __forceinline__ void tmaStoreRow(uint32_t src, uint32_t N, const float* bias, int act,
                                            unsigned char* buf, uint32_t accEmptyBar, const CUtensorMap* mapOut,
                                            int cx, int px0, int py, int img) {
    const uint32_t lane = threadIdx.x & 31u;
    if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 1;\n" ::: "memory");
    __syncwarp();
    const uint32_t rowBytes = 2u * N;
    const uint32_t swzMask = (rowBytes >> 4) - 1u;                          // 16-byte chunks per row - 1
    const uint32_t f = ((lane * rowBytes) >> 7) & swzMask;                  // address bits 7.. of the row
    const bool biasVec = bias && (reinterpret_cast<uintptr_t>(bias) & 15u) == 0u;
    for (uint32_t c = 0; c < N; c += 16u) {
        uint32_t rr[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
            "%12, %13, %14, %15}, [%16];\n"
            : "=r"(rr[0]), "=r"(rr[1]), "=r"(rr[2]), "=r"(rr[3]), "=r"(rr[4]), "=r"(rr[5]), "=r"(rr[6]), "=r"(rr[7]),
              "=r"(rr[8]), "=r"(rr[9]), "=r"(rr[10]), "=r"(rr[11]), "=r"(rr[12]), "=r"(rr[13]), "=r"(rr[14]),
              "=r"(rr[15])
            : "r"(src + c));
        float bv[16];
        if (biasVec) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float4 b4 = __ldg(reinterpret_cast<const float4*>(bias + c) + k);
                bv[4 * k] = b4.x;
                bv[4 * k + 1] = b4.y;
                bv[4 * k + 2] = b4.z;
                bv[4 * k + 3] = b4.w;
            }
        } else {
#pragma unroll
            for (int k = 0; k < 16; ++k) bv[k] = bias ? __ldg(bias + c + k) : 0.0f;
        }
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        uint32_t packed[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            float x0 = __uint_as_float(rr[2 * k]), x1 = __uint_as_float(rr[2 * k + 1]);
            if (bias) {
                x0 += bv[2 * k];
                x1 += bv[2 * k + 1];
            }
            if (act == 1) {
                x0 = fmaxf(x0, 0.0f);
                x1 = fmaxf(x1, 0.0f);
            }
            __nv_bfloat162 h2 = __floats2bfloat162_rn(x0, x1);
            packed[k] = *reinterpret_cast<uint32_t*>(&h2);
        }
        const uint32_t j = c >> 3;  // first 16-byte chunk of these 16 channels
        unsigned char* row = buf + lane * rowBytes;
        *reinterpret_cast<uint4*>(row + (((j) ^ f) << 4)) = make_uint4(packed[0], packed[1], packed[2], packed[3]);
        *reinterpret_cast<uint4*>(row + (((j + 1u) ^ f) << 4)) = make_uint4(packed[4], packed[5], packed[6], packed[7]);
    }
    zeroColumns(src, 0u, N);  // the next row in this accumulator slot starts from zero
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    mbarArrive(accEmptyBar);
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // the box is visible to the copy engine
    __syncwarp();
    if (lane == 0) {
        asm volatile(
            "cp.async.bulk.tensor.4d.global.shared::cta.bulk_group [%0, {%1, %2, %3, %4}], [%5];\n" ::"l"(mapOut),
            "r"(cx), "r"(px0), "r"(py), "r"(img), "r"(smemAddr(buf))
            : "memory");
        asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
    }
}

// The 2x2 average of the two rows a warp has just staged for tensor stores
// (`top`: row 2i, `bottom`: row 2i + 1; 32 pixels x N channels each, laid out
// as in tmaStoreRow): lane l takes pooled pixel l / 2 and half of its
// channels and writes them to `dst` (that pooled pixel's first channel, or
// null past the image's right edge).  The staged values are the output's
// bf16 bits, and the sum ((top-left + top-right) + bottom-left) +
// bottom-right, times 0.25, is the pooling kernel's own, so the result is the
// one a separate pooling pass over the stored output gives.  The boxes were
// written before the warp's last __syncwarp in tmaStoreRow; they are next
// overwritten after the next one.
__device__ __forceinline__ void poolPairRow(const unsigned char* top, const unsigned char* bottom, uint32_t N,
                                            __nv_bfloat16* dst) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t rowBytes = 2u * N, swzMask = (rowBytes >> 4) - 1u;
    const uint32_t left = lane & ~1u, right = left + 1u;
    const uint32_t fl = ((left * rowBytes) >> 7) & swzMask, fr = ((right * rowBytes) >> 7) & swzMask;
    const uint32_t per = N >> 4;  // 16-byte chunks (8 channels) per lane
    const uint32_t j0 = (lane & 1u) * per;
    for (uint32_t j = j0; j < j0 + per; ++j) {
        const uint4 tl = *reinterpret_cast<const uint4*>(top + left * rowBytes + ((j ^ fl) << 4));
        const uint4 tr = *reinterpret_cast<const uint4*>(top + right * rowBytes + ((j ^ fr) << 4));
        const uint4 bl = *reinterpret_cast<const uint4*>(bottom + left * rowBytes + ((j ^ fl) << 4));
        const uint4 br = *reinterpret_cast<const uint4*>(bottom + right * rowBytes + ((j ^ fr) << 4));
        const uint32_t a[4] = {tl.x, tl.y, tl.z, tl.w}, b[4] = {tr.x, tr.y, tr.z, tr.w};
        const uint32_t c[4] = {bl.x, bl.y, bl.z, bl.w}, d[4] = {br.x, br.y, br.z, br.w};
        uint32_t o[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float2 s = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&a[k]));
            const float2 t = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&b[k]));
            const float2 u = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&c[k]));
            const float2 v = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&d[k]));
            __nv_bfloat162 h2 = __floats2bfloat162_rn(0.25f * (s.x + t.x + u.x + v.x), 0.25f * (s.y + t.y + u.y + v.y));
            o[k] = *reinterpret_cast<uint32_t*>(&h2);
        }
        if (dst) *reinterpret_cast<uint4*>(dst + 8u * j) = make_uint4(o[0], o[1], o[2], o[3]);
    }
}

// A run of output rows y0..y1-1 of tile column tx of image img.
struct RowSegment {
    uint32_t img, tx, y0, y1;
};
// The next segment of this CTA's rows [cur, end): the rest of the current
// tile column at most; false when the range is done.
__device__ __forceinline__ bool nextSegment(const HaloConvArgs& a, uint32_t& cur, uint32_t end, RowSegment& sg) {
    if (cur >= end) return false;
    const uint32_t col = cur / a.h;
    sg.y0 = cur - col * a.h;
    sg.y1 = min(a.h, sg.y0 + (end - cur));
    sg.tx = col % a.tilesX;
    sg.img = col / a.tilesX;
    cur += sg.y1 - sg.y0;
    return true;
}
// With pooling (h even), ranges hold whole row pairs, so that rows 2i and
// 2i + 1 of a tile column reach the same epilogue set one after the other.
__device__ __forceinline__ uint32_t rangeBegin(const HaloConvArgs& a, uint32_t cta) {
    if (a.pool) return 2u * (uint32_t)((uint64_t)cta * (a.totalRows >> 1) / gridDim.x);
    return (uint32_t)((uint64_t)cta * a.totalRows / gridDim.x);
}

// kC: 64-channel chunks of the input (Cin / 64 rounded up), kLast: K steps of
// 16 channels in the last chunk.  Both are compile-time so that each output
// row's MMAs are straight-line code: a branch between two tcgen05.mma costs
// the issuing thread a few hundred cycles (measured), about the time of a
// 128 x 32 x 16 MMA twenty times over.
template <bool kStack, uint32_t kC, uint32_t kLast>
__global__ void __launch_bounds__(320, 1)
    k_conv3x3_halo(const __grid_constant__ CUtensorMap mapIn, const __grid_constant__ CUtensorMap mapW,
                   const __grid_constant__ CUtensorMap mapOut, HaloConvArgs a) {
    extern __shared__ unsigned char dsm[];
    const uint32_t raw = smemAddr(dsm);
    unsigned char* sm = dsm + (((raw + 1023u) & ~1023u) - raw);
    const uint32_t N = a.cout, C = a.chunks;
    const uint32_t slotBytes = C * kHaloSlotBytes;
    const uint32_t wBoxBytes = N * 128u, wBytes = 9u * C * wBoxBytes;
    unsigned char* sRing = sm;
    const uint32_t R = a.ring;
    unsigned char* sW = sm + R * slotBytes;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sW + wBytes);
    // bars: full[R], empty[R], weights, accFull[Q], accEmpty[Q]
    const uint32_t fullBar = smemAddr(bars), emptyBar = fullBar + 8u * kHaloRingMax;
    const uint32_t wBar = emptyBar + 8u * kHaloRingMax, accFullBar = wBar + 8u;
    const uint32_t accEmptyBar = accFullBar + 8u * kHaloAccMax;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2 * kHaloRingMax + 1 + 2 * kHaloAccMax);
    // Accumulators: Q slots of Cout columns for the stacked variant (a rolling
    // window over the output rows), else nbuf buffers of `cols` columns.
    const uint32_t nbuf = kStack ? a.slots : accBuffers(a.cols);
    const uint32_t bufShift = kStack ? a.logSlots : (nbuf == 4u ? 2u : 1u);
    const uint32_t tmemCols = kStack ? 512u : nbuf * a.cols;
    int* abortFlag = reinterpret_cast<int*>(tslot + 1);
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;

    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smemAddr(tslot)),
                     "r"(tmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    if (tid == 0) {
        for (uint32_t s = 0; s < R; ++s) {
            mbarInit(fullBar + 8u * s, 1);
            mbarInit(emptyBar + 8u * s, 1);
        }
        mbarInit(wBar, 1);
        for (uint32_t b = 0; b < nbuf; ++b) {
            mbarInit(accFullBar + 8u * b, 1);
            mbarInit(accEmptyBar + 8u * b, (kStack || !epiSplit(N)) ? 128u : 256u);
        }
        *abortFlag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(&mapIn) : "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"(&mapW) : "memory");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    pdlRelease();
    pdlWait();
    const uint32_t taddr = *tslot;
    volatile int* abortV = abortFlag;

    if (warp == 0) {
        if (lane == 0) {
            mbarExpectTx(wBar, wBytes);
            // Stacked: per (dx, chunk) one tile of 3 x Cout weight rows, the taps
            // dy = 2, 1, 0 in that order (an MMA with N = 3 Cout then yields the
            // contributions of one halo row to output rows y - 2, y - 1, y).
            for (uint32_t tap = 0; tap < 9u; ++tap)
                for (uint32_t c = 0; c < C; ++c) {
                    const uint32_t dy = tap / 3u, dx = tap - 3u * dy;
                    const uint32_t box = kStack ? (dx * C + c) * 3u + (2u - dy) : tap * C + c;
                    tmaLoad3(smemAddr(sW + box * wBoxBytes), &mapW, (int)(c * 64u), (int)tap, 0, wBar);
                }
            uint32_t g = 0;
            RingPos pos{0u, 0u};
            uint32_t cur = rangeBegin(a, blockIdx.x);
            const uint32_t end = rangeBegin(a, blockIdx.x + 1u);
            RowSegment sg;
            while (!*abortV && nextSegment(a, cur, end, sg)) {
                const int x0 = (int)(sg.tx * 128u), y0 = (int)sg.y0, y1 = (int)sg.y1;
                const uint32_t img = sg.img;
                bool ok = true;
                for (int hy = y0 - 1; hy <= y1; ++hy, ++g, pos.advance(R)) {
                    if (g >= R && !mbarWait(emptyBar + 8u * pos.slot, pos.phase ^ 1u)) {
                        ok = false;
                        break;
                    }
                    const uint32_t full = fullBar + 8u * pos.slot;
                    mbarExpectTx(full, C * kHaloPix * 128u);
                    for (uint32_t c = 0; c < C; ++c)
                        tmaLoad4(smemAddr(sRing + pos.slot * slotBytes + c * kHaloSlotBytes), &mapIn, (int)(c * 64u),
                                 x0 - 1, hy, (int)img, full);
                }
                if (!ok) {
                    *abortV = 1;
                    break;
                }
            }
        }
    } else if (warp == 1 && kStack) {
        if (lane == 0) {
            // Per halo row k of a segment of `rows` output rows: the row's
            // contributions to output rows k - 2, k - 1, k (taps dy = 2, 1, 0).
            // Between the segment's edges, and when the three rows' slots are
            // adjacent, that is one MMA per (dx, chunk, K step) with N = 3 Cout
            // into the three slots; otherwise one MMA with N = Cout per valid
            // row.  Slots start zeroed (the epilogue clears a slot when it has
            // read it), so every MMA accumulates.
            const uint32_t idesc1 = (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((128u >> 4) << 24);
            const uint32_t idesc3 = (1u << 4) | (1u << 7) | (1u << 10) | (((3u * N) >> 3) << 17) | ((128u >> 4) << 24);
            const uint32_t hi = descHi(), aLo0 = descLo(smemAddr(sRing)), bLo0 = descLo(smemAddr(sW));
            const uint32_t tileU = (3u * wBoxBytes) >> 4, dyU = wBoxBytes >> 4;  // in 16-byte units
            const uint32_t Q = nbuf;
            // One halo row's stacked MMAs (N = 3 Cout) into the slots from `d` on.
            auto stackedRow = [&](uint32_t aRow, uint32_t d) {
#pragma unroll
                for (uint32_t dx = 0; dx < 3u; ++dx)
#pragma unroll
                    for (uint32_t c = 0; c < kC; ++c)
#pragma unroll
                        for (uint32_t ks = 0; ks < (c + 1u < kC ? 4u : kLast); ++ks)
                            mmaF16(d, aRow + dx * 8u + c * (kHaloSlotBytes >> 4) + 2u * ks,  // pixel dx: 128 B on
                                   bLo0 + (dx * kC + c) * tileU + 2u * ks, hi, idesc3, 1u);
            };
            bool ok = mbarWait(wBar, 0u);
            uint32_t t0 = 0;      // output rows of the earlier segments
            RingPos hp{0u, 0u};   // the current halo row's ring slot
            uint32_t cur = rangeBegin(a, blockIdx.x);
            const uint32_t end = rangeBegin(a, blockIdx.x + 1u);
            RowSegment sg;
            while (ok && !*abortV && nextSegment(a, cur, end, sg)) {
                const uint32_t rows = sg.y1 - sg.y0;
                for (uint32_t k = 0; k < rows + 2u;) {
                    // Two interior halo rows at once when both stack into adjacent
                    // slots: their waits first, then both rows' MMAs and commits as
                    // one straight-line run (one branch per two rows).
                    if (k >= 2u && k + 1u < rows && ((t0 + k - 2u) & (Q - 1u)) + 3u < Q) {
                        RingPos hp1 = hp;
                        hp1.advance(R);
                        const uint32_t t = t0 + k, sLo = (t0 + k - 2u) & (Q - 1u);
                        if (!mbarWait(accEmptyBar + 8u * (t & (Q - 1u)), (t >> bufShift) & 1u) ||
                            !mbarWait(accEmptyBar + 8u * ((t + 1u) & (Q - 1u)), ((t + 1u) >> bufShift) & 1u) ||
                            !mbarWait(fullBar + 8u * hp.slot, hp.phase) || !mbarWait(fullBar + 8u * hp1.slot, hp1.phase)) {
                            ok = false;
                            break;
                        }
                        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                        stackedRow(aLo0 + hp.slot * (slotBytes >> 4), taddr + sLo * N);
                        umaCommit(emptyBar + 8u * hp.slot);
                        umaCommit(accFullBar + 8u * sLo);
                        stackedRow(aLo0 + hp1.slot * (slotBytes >> 4), taddr + (sLo + 1u) * N);
                        umaCommit(emptyBar + 8u * hp1.slot);
                        umaCommit(accFullBar + 8u * (sLo + 1u));
                        k += 2u;
                        hp = hp1;
                        hp.advance(R);
                        continue;
                    }
                    if (k < rows) {  // output row k enters: its slot must have been read and cleared
                        const uint32_t t = t0 + k;
                        if (!mbarWait(accEmptyBar + 8u * (t & (Q - 1u)), (t >> bufShift) & 1u)) ok = false;
                    }
                    if (ok && !mbarWait(fullBar + 8u * hp.slot, hp.phase)) ok = false;
                    if (!ok) break;
                    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                    const uint32_t aRow = aLo0 + hp.slot * (slotBytes >> 4);
                    const uint32_t jLo = k >= 2u ? k - 2u : 0u, jHi = min(k, rows - 1u);
                    const uint32_t sLo = (t0 + jLo) & (Q - 1u);
                    const bool stacked = k >= 2u && k < rows && sLo + 2u < Q;
                    if (stacked) {
                        stackedRow(aRow, taddr + sLo * N);
                    } else {
                        for (uint32_t j = jLo; j <= jHi; ++j) {
                            const uint32_t dy = k - j;
                            const uint32_t d = taddr + ((t0 + j) & (Q - 1u)) * N;
#pragma unroll
                            for (uint32_t dx = 0; dx < 3u; ++dx)
#pragma unroll
                                for (uint32_t c = 0; c < kC; ++c)
#pragma unroll
                                    for (uint32_t ks = 0; ks < (c + 1u < kC ? 4u : kLast); ++ks)
                                        mmaF16(d, aRow + dx * 8u + c * (kHaloSlotBytes >> 4) + 2u * ks,
                                               bLo0 + (dx * kC + c) * tileU + (2u - dy) * dyU + 2u * ks, hi, idesc1,
                                               1u);
                        }
                    }
                    umaCommit(emptyBar + 8u * hp.slot);  // halo row k has no reader left
                    if (k >= 2u) umaCommit(accFullBar + 8u * ((t0 + k - 2u) & (Q - 1u)));  // row k - 2 is complete
                    ++k;
                    hp.advance(R);
                }
                t0 += rows;
            }
            if (!ok) *abortV = 1;
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((128u >> 4) << 24);
            const uint32_t hi = descHi(), aLo0 = descLo(smemAddr(sRing)), bLo0 = descLo(smemAddr(sW));
            bool ok = mbarWait(wBar, 0u);
            uint32_t t = 0;
            RingPos top{0u, 0u};  // the item's first halo row
            uint32_t cur = rangeBegin(a, blockIdx.x);
            const uint32_t end = rangeBegin(a, blockIdx.x + 1u);
            RowSegment sg;
            while (ok && !*abortV && nextSegment(a, cur, end, sg)) {
                const uint32_t rows = sg.y1 - sg.y0;
                // halo rows w0, w1, w2 feed the current output row
                RingPos w0 = top, w1 = top, w2;
                w1.advance(R);
                w2 = w1;
                w2.advance(R);
                if (!mbarWait(fullBar + 8u * w0.slot, w0.phase) || !mbarWait(fullBar + 8u * w1.slot, w1.phase))
                    ok = false;
                for (uint32_t k = 0; ok && k < rows; ++k, ++t) {
                    if (!mbarWait(fullBar + 8u * w2.slot, w2.phase)) ok = false;
                    const uint32_t b = t & (nbuf - 1u), v = t >> bufShift;
                    if (ok && v > 0 && !mbarWait(accEmptyBar + 8u * b, (v - 1u) & 1u)) ok = false;
                    if (!ok) break;
                    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                    const uint32_t dAddr = taddr + b * a.cols;
                    // A run that starts inside the 1024-byte swizzle pattern (pixel dx)
                    // takes the plain descriptor: the tensor core applies the 128-byte
                    // swizzle to absolute shared-memory address bits, as the copy engine
                    // wrote it (measured: a base offset of (start >> 7) & 7 gives wrong sums).
                    const uint32_t rowLo[3] = {aLo0 + w0.slot * (slotBytes >> 4), aLo0 + w1.slot * (slotBytes >> 4),
                                               aLo0 + w2.slot * (slotBytes >> 4)};
#pragma unroll
                    for (uint32_t tap = 0; tap < 9u; ++tap) {
                        const uint32_t dy = tap / 3u, dx = tap - dy * 3u;
                        const uint32_t aT = rowLo[dy] + dx * 8u;  // pixel dx: 128 bytes further
                        const uint32_t bT = bLo0 + tap * kC * (wBoxBytes >> 4);
#pragma unroll
                        for (uint32_t c = 0; c < kC; ++c)
#pragma unroll
                            for (uint32_t ks = 0; ks < (c + 1u < kC ? 4u : kLast); ++ks)
                                mmaF16(dAddr, aT + c * (kHaloSlotBytes >> 4) + 2u * ks, bT + c * (wBoxBytes >> 4) + 2u * ks,
                                       hi, idesc, (tap | c | ks) ? 1u : 0u);
                    }
                    umaCommit(accFullBar + 8u * b);          // output row complete
                    umaCommit(emptyBar + 8u * w0.slot);      // its top halo row has no reader left
                    w0 = w1;
                    w1 = w2;
                    w2.advance(R);
                }
                if (!ok) break;
                umaCommit(emptyBar + 8u * w0.slot);  // the item's last two halo rows
                umaCommit(emptyBar + 8u * w1.slot);
                top = w2;
            }
            if (!ok) *abortV = 1;
        }
    } else {
        // Epilogue warps 2..9: TMEM lane quarter warp % 4 (one output pixel per
        // thread); set (warp - 2) / 4.  Stacked: set s takes every channel of
        // the rows of parity s (and owns the accumulator slots of that parity:
        // the slot count is even), two rows in flight -- with pooling, of the
        // row pairs of parity s (slot count a multiple of 4); otherwise both
        // sets take every row, each half of the channels.
        const uint32_t q = warp & 3u, set = (warp - 2u) >> 2;
        const uint32_t r = q * 32u + lane;
        const uint32_t cw = epiCols(N);
        const uint32_t c0 = kStack ? 0u : set * cw, c1 = kStack ? N : (epiSplit(N) ? c0 + cw : (set ? 0u : N));
        unsigned char* stage = a.staged ? reinterpret_cast<unsigned char*>(bars) + kHaloBarBytes +
                                              (warp - 2u) * (kStack ? epiWarpBytesAll(N) : epiWarpBytes(N))
                                        : nullptr;
        uint32_t t = 0;
        bool ok = c1 > c0;
        const uint32_t quarter = taddr + ((q * 32u) << 16);
        const uint32_t slotCols = kStack ? N : a.cols;
        const uint32_t pairShift = a.pool ? 1u : 0u;  // rows (or row pairs) alternate between the sets
        if (kStack) {
            // Every slot starts zeroed; its first release lets the MMA warp in.
            for (uint32_t b = 0; b < nbuf; ++b)
                if (((b >> pairShift) & 1u) == set) zeroColumns(quarter + b * slotCols, c0, c1);
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            for (uint32_t b = 0; b < nbuf; ++b)
                if (((b >> pairShift) & 1u) == set) mbarArrive(accEmptyBar + 8u * b);
        }
        uint32_t cur = rangeBegin(a, blockIdx.x);
        const uint32_t end = rangeBegin(a, blockIdx.x + 1u);
        RowSegment sg;
        // Stacked with TMA stores: two boxes of 32 pixels x N channels per warp.
        unsigned char* boxes = reinterpret_cast<unsigned char*>(bars) + kHaloBarBytes + (warp - 2u) * 128u * N;
        uint32_t stored = 0;
        while (ok && nextSegment(a, cur, end, sg)) {
            const uint32_t img = sg.img, px = sg.tx * 128u + r;
            for (uint32_t py = sg.y0; py < sg.y1; ++py, ++t) {
                if (kStack && ((t >> pairShift) & 1u) != set) continue;  // the other set's row
                if (kStack && a.tmaStore) {
                    const uint32_t b = t & (nbuf - 1u), v = t >> bufShift;
                    if (!mbarWait(accFullBar + 8u * b, v & 1u)) {
                        *abortV = 1;
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                    const uint32_t box = stored & 1u;
                    tmaStoreRow(quarter + b * slotCols, N, a.bias, a.act, boxes + box * 64u * N, accEmptyBar + 8u * b,
                                &mapOut, (int)a.coOff, (int)(sg.tx * 128u + q * 32u), (int)py, (int)img);
                    ++stored;
                    if (a.pool && (py & 1u)) {  // rows py - 1 and py are in this warp's two boxes
                        const uint32_t left = sg.tx * 128u + q * 32u + (lane & ~1u);
                        __nv_bfloat16* dst =
                            left < a.w ? a.pool + ((size_t)(img * (a.h >> 1) + (py >> 1)) * (a.w >> 1) + (left >> 1)) *
                                                      a.poolLd
                                       : nullptr;
                        poolPairRow(boxes + (box ^ 1u) * 64u * N, boxes + box * 64u * N, N, dst);
                    }
                    continue;
                }
                const uint32_t b = t & (nbuf - 1u), v = t >> bufShift;
                if (!mbarWait(accFullBar + 8u * b, v & 1u)) {
                    *abortV = 1;
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                __nv_bfloat16* orow =
                    px < a.w ? a.out + ((size_t)(img * a.h + py) * a.w + px) * a.ldo + a.coOff : nullptr;
                epilogueRow(quarter + b * slotCols, c0, c1, a.bias, a.act, a.accumulate, orow, stage,
                            accEmptyBar + 8u * b, kStack);
            }
        }
        if (kStack && a.tmaStore && lane == 0) asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
    }
    __syncthreads();
    if (*abortV && tid == 0) atomicExch(&g_unetError, 3);
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(tmemCols));
}

size_t haloSmemBytes(uint32_t cout, uint32_t chunks, bool staged, uint32_t ring, bool stack, bool tmaStore = false) {
    const size_t epi = tmaStore ? kEpiWarps * 128u * cout  // two boxes of 32 pixels x Cout per warp
                                : (staged ? kEpiWarps * (stack ? epiWarpBytesAll(cout) : epiWarpBytes(cout)) : 0u);
    return 1024u + (size_t)ring * chunks * kHaloSlotBytes + 9u * (size_t)chunks * cout * 128u + kHaloBarBytes + epi;
}

// -------------------------------------------------------------- wgrad ----
struct WgradArgs {
    const __nv_bfloat16* in;    // [M][ldi], channels [0, cin)
    const __nv_bfloat16* dout;  // [M][ldd], channels [0, cout)
    float* dw;                  // [cout][9][cin], accumulated
    uint32_t n, h, w_, cin, ldi, cout, ldd, M;
    uint32_t chunk;             // pixels per block (multiple of 32)
};

constexpr int kWB = 64;  // co and ci per block

// Byte offset of 16-byte chunk `seg` (0..7) of row `r` in a 128-byte-row tile.
__device__ __forceinline__ uint32_t swz128(uint32_t r, uint32_t seg) { return r * 128u + ((seg ^ (r & 7u)) << 4); }

__global__ void __launch_bounds__(128) k_conv3x3_wgrad(WgradArgs a) {
    __shared__ __align__(128) unsigned char sA[2][32 * 128];  // [pixel][64 co]
    __shared__ __align__(128) unsigned char sB[2][32 * 128];  // [pixel][64 ci]
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t tap = blockIdx.z;
    const uint32_t ciTiles = (a.cin + kWB - 1) / kWB;
    const uint32_t co0 = (blockIdx.y / ciTiles) * kWB, ci0 = (blockIdx.y % ciTiles) * kWB;
    const uint32_t p0 = blockIdx.x * a.chunk, p1 = min(p0 + a.chunk, a.M);
    const int dy = (int)(tap / 3u) - 1, dx = (int)(tap % 3u) - 1;
    const uint32_t HW = a.h * a.w_;
    const uint32_t wm = warp >> 1, wn = warp & 1u;  // 2 x 2 warps of 32 co x 32 ci

    auto loadStage = [&](uint32_t pb, int stage) {
        // 32 pixels x 8 chunks for each operand: 2 + 2 chunks per thread.
#pragma unroll
        for (uint32_t k = 0; k < 2; ++k) {
            uint32_t i = tid + k * 128u, row = i >> 3, seg = i & 7u;
            uint32_t p = pb + row;
            bool pv = p < p1;
            bool v = pv && co0 + seg * 8u < a.cout;
            const __nv_bfloat16* src = a.dout + (size_t)p * a.ldd + co0 + seg * 8u;
            cpAsync16(&sA[stage][swz128(row, seg)], v ? src : a.dout, v ? 16u : 0u);
            bool vb = false;
            const __nv_bfloat16* bsrc = a.in;
            if (pv && ci0 + seg * 8u < a.cin) {
                uint32_t img = p / HW, rem = p - img * HW;
                int yy = (int)(rem / a.w_) + dy, xx = (int)(rem % a.w_) + dx;
                if (yy >= 0 && yy < (int)a.h && xx >= 0 && xx < (int)a.w_) {
                    vb = true;
                    bsrc = a.in + ((size_t)(img * a.h + (uint32_t)yy) * a.w_ + (uint32_t)xx) * a.ldi + ci0 + seg * 8u;
                }
            }
            cpAsync16(&sB[stage][swz128(row, seg)], bsrc, vb ? 16u : 0u);
        }
    };

    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.0f;

    const uint32_t steps = (p1 > p0) ? (p1 - p0 + 31u) / 32u : 0u;
    if (steps > 0) loadStage(p0, 0);
    cpAsyncCommit();
    for (uint32_t s = 0; s < steps; ++s) {
        if (s + 1 < steps) loadStage(p0 + (s + 1) * 32u, (int)((s + 1) & 1u));
        cpAsyncCommit();
        cpAsyncWait<1>();
        __syncthreads();
        const int st = (int)(s & 1u);
#pragma unroll
        for (uint32_t kk = 0; kk < 2; ++kk) {  // 16 pixels each
            uint32_t af[2][4];
#pragma unroll
            for (uint32_t mt = 0; mt < 2; ++mt) {
                // A (co x p) from sA[p][co] through transposed 8x8 loads:
                // matrices (co 0-7, p 0-7), (co 8-15, p 0-7), (co 0-7, p 8-15), (co 8-15, p 8-15).
                uint32_t id = lane >> 3;
                uint32_t prow = kk * 16u + ((id >> 1) << 3) + (lane & 7u);
                uint32_t seg = (wm * 32u + mt * 16u) / 8u + (id & 1u);
                ldmatrixX4T(af[mt][0], af[mt][1], af[mt][2], af[mt][3], &sA[st][swz128(prow, seg)]);
            }
#pragma unroll
            for (uint32_t np = 0; np < 2; ++np) {
                // B (p x ci): matrices (p 0-7, ci 0-7), (p 8-15, ci 0-7), (p 0-7, ci 8-15), (p 8-15, ci 8-15).
                uint32_t id = lane >> 3;
                uint32_t prow = kk * 16u + ((id & 1u) << 3) + (lane & 7u);
                uint32_t seg = (wn * 32u + np * 16u) / 8u + (id >> 1);
                uint32_t b0, b1, b2, b3;
                ldmatrixX4T(b0, b1, b2, b3, &sB[st][swz128(prow, seg)]);
#pragma unroll
                for (uint32_t mt = 0; mt < 2; ++mt) {
                    mmaBf16(acc[mt][2 * np], af[mt], b0, b1);
                    mmaBf16(acc[mt][2 * np + 1], af[mt], b2, b3);
                }
            }
        }
        __syncthreads();
    }
    cpAsyncWait<0>();
#pragma unroll
    for (uint32_t mt = 0; mt < 2; ++mt)
#pragma unroll
        for (uint32_t half = 0; half < 2; ++half) {
            uint32_t co = co0 + wm * 32u + mt * 16u + (lane >> 2) + half * 8u;
            if (co >= a.cout) continue;
#pragma unroll
            for (uint32_t nt = 0; nt < 4; ++nt) {
                uint32_t ci = ci0 + wn * 32u + nt * 8u + (lane & 3u) * 2u;
                if (ci >= a.cin) continue;
                float* dst = a.dw + ((size_t)co * 9u + tap) * a.cin + ci;
                atomicAdd(dst, acc[mt][nt][half * 2 + 0]);
                atomicAdd(dst + 1, acc[mt][nt][half * 2 + 1]);
            }
        }
}

// ------------------------------------------------------- elementwise ----
__device__ __forceinline__ uint32_t gid() { return blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ uint32_t gstride() { return gridDim.x * blockDim.x; }

// dPre = dOut where out > 0 (ReLU), over `c` channels of every pixel.
__global__ void k_relu_backward(const __nv_bfloat16* out, uint32_t ldo, const __nv_bfloat16* dout, uint32_t ldd,
                                __nv_bfloat16* dpre, uint32_t ldp, uint32_t c, uint32_t M) {
    const uint32_t pairs = c / 2u;
    for (uint64_t i = gid(); i < (uint64_t)M * pairs; i += gstride()) {
        uint32_t p = (uint32_t)(i / pairs), k = (uint32_t)(i % pairs) * 2u;
        __nv_bfloat162 o = *reinterpret_cast<const __nv_bfloat162*>(out + (size_t)p * ldo + k);
        __nv_bfloat162 d = *reinterpret_cast<const __nv_bfloat162*>(dout + (size_t)p * ldd + k);
        float2 of = __bfloat1622float2(o), df = __bfloat1622float2(d);
        *reinterpret_cast<__nv_bfloat162*>(dpre + (size_t)p * ldp + k) =
            __floats2bfloat162_rn(of.x > 0.0f ? df.x : 0.0f, of.y > 0.0f ? df.y : 0.0f);
    }
}

// Per-channel sums of dPre (the bias gradient), accumulated into db.
__global__ void k_bias_grad(const __nv_bfloat16* dpre, uint32_t ld, uint32_t c, uint32_t M, float* db) {
    // blockDim.x = 256: thread handles channel (tid % c) over a pixel stripe.
    __shared__ float partial[256];
    uint32_t ch = threadIdx.x % c, lanes = 256u / c;
    uint32_t lanePix = threadIdx.x / c;
    float s = 0.0f;
    if (lanePix < lanes)
        for (uint32_t p = blockIdx.x * lanes + lanePix; p < M; p += gridDim.x * lanes)
            s += __bfloat162float(dpre[(size_t)p * ld + ch]);
    partial[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x < c) {
        float t = 0.0f;
        for (uint32_t k = 0; k < lanes; ++k) t += partial[k * c + threadIdx.x];
        atomicAdd(&db[threadIdx.x], t);
    }
}

// 2x2 average pooling: out (h/2, w/2).
__global__ void k_avgpool2(const __nv_bfloat16* in, uint32_t ldi, __nv_bfloat16* out, uint32_t ldo, uint32_t coOff,
                           uint32_t c, uint32_t n, uint32_t h, uint32_t w) {
    const uint32_t ho = h / 2u, wo = w / 2u, pairs = c / 2u;
    for (uint64_t i = gid(); i < (uint64_t)n * ho * wo * pairs; i += gstride()) {
        uint32_t k = (uint32_t)(i % pairs) * 2u;
        uint64_t q = i / pairs;
        uint32_t x = (uint32_t)(q % wo), y = (uint32_t)((q / wo) % ho), b = (uint32_t)(q / ((uint64_t)wo * ho));
        size_t base = ((size_t)(b * h + 2u * y) * w + 2u * x) * ldi + k;
        float2 s = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(in + base));
        float2 t = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(in + base + ldi));
        float2 u = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(in + base + (size_t)w * ldi));
        float2 v = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(in + base + (size_t)w * ldi + ldi));
        *reinterpret_cast<__nv_bfloat162*>(out + q * ldo + coOff + k) =
            __floats2bfloat162_rn(0.25f * (s.x + t.x + u.x + v.x), 0.25f * (s.y + t.y + u.y + v.y));
    }
}

// Gradient of the 2x2 average pool: din (+)= dout / 4 on each of the 4 inputs.
__global__ void k_avgpool2_backward(const __nv_bfloat16* dout, uint32_t ldd, __nv_bfloat16* din, uint32_t ldi,
                                    uint32_t c, uint32_t n, uint32_t h, uint32_t w, int accumulate) {
    const uint32_t wo = w / 2u, pairs = c / 2u;
    for (uint64_t i = gid(); i < (uint64_t)n * h * w * pairs; i += gstride()) {
        uint32_t k = (uint32_t)(i % pairs) * 2u;
        uint64_t q = i / pairs;
        uint32_t x = (uint32_t)(q % w), y = (uint32_t)((q / w) % h), b = (uint32_t)(q / ((uint64_t)w * h));
        float2 d = __bfloat1622float2(
            *reinterpret_cast<const __nv_bfloat162*>(dout + ((size_t)(b * (h / 2u) + y / 2u) * wo + x / 2u) * ldd + k));
        __nv_bfloat162* dst = reinterpret_cast<__nv_bfloat162*>(din + q * ldi + k);
        float2 v = make_float2(0.25f * d.x, 0.25f * d.y);
        if (accumulate) {
            float2 o = __bfloat1622float2(*dst);
            v.x += o.x;
            v.y += o.y;
        }
        *dst = __floats2bfloat162_rn(v.x, v.y);
    }
}

// Nearest 2x upsampling: out (2h, 2w).
__global__ void k_upsample2(const __nv_bfloat16* in, uint32_t ldi, __nv_bfloat16* out, uint32_t ldo, uint32_t coOff,
                            uint32_t c, uint32_t n, uint32_t h, uint32_t w) {
    const uint32_t H = 2u * h, W = 2u * w, pairs = c / 2u;
    for (uint64_t i = gid(); i < (uint64_t)n * H * W * pairs; i += gstride()) {
        uint32_t k = (uint32_t)(i % pairs) * 2u;
        uint64_t q = i / pairs;
        uint32_t x = (uint32_t)(q % W), y = (uint32_t)((q / W) % H), b = (uint32_t)(q / ((uint64_t)W * H));
        *reinterpret_cast<__nv_bfloat162*>(out + q * ldo + coOff + k) =
            *reinterpret_cast<const __nv_bfloat162*>(in + ((size_t)(b * h + y / 2u) * w + x / 2u) * ldi + k);
    }
}

// Gradient of the nearest upsampling: din = sum of the 4 output gradients.
__global__ void k_upsample2_backward(const __nv_bfloat16* dout, uint32_t ldd, uint32_t ciOff, __nv_bfloat16* din,
                                     uint32_t ldi, uint32_t c, uint32_t n, uint32_t h, uint32_t w) {
    const uint32_t W = 2u * w, pairs = c / 2u;
    for (uint64_t i = gid(); i < (uint64_t)n * h * w * pairs; i += gstride()) {
        uint32_t k = (uint32_t)(i % pairs) * 2u;
        uint64_t q = i / pairs;
        uint32_t x = (uint32_t)(q % w), y = (uint32_t)((q / w) % h), b = (uint32_t)(q / ((uint64_t)w * h));
        size_t base = ((size_t)(b * 2u * h + 2u * y) * W + 2u * x) * ldd + ciOff + k;
        float2 s = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(dout + base));
        float2 t = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(dout + base + ldd));
        float2 u = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(dout + base + (size_t)W * ldd));
        float2 v = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(dout + base + (size_t)W * ldd + ldd));
        *reinterpret_cast<__nv_bfloat162*>(din + q * ldi + k) =
            __floats2bfloat162_rn(s.x + t.x + u.x + v.x, s.y + t.y + u.y + v.y);
    }
}

// Channel-slice copy (skip connections into concat buffers, gradient routing).
__global__ void k_copy_channels(const __nv_bfloat16* src, uint32_t lds, uint32_t sOff, __nv_bfloat16* dst,
                                uint32_t ldd, uint32_t dOff, uint32_t c, uint32_t M, int accumulate) {
    const uint32_t pairs = c / 2u;
    for (uint64_t i = gid(); i < (uint64_t)M * pairs; i += gstride()) {
        uint32_t p = (uint32_t)(i / pairs), k = (uint32_t)(i % pairs) * 2u;
        float2 v = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(src + (size_t)p * lds + sOff + k));
        __nv_bfloat162* d = reinterpret_cast<__nv_bfloat162*>(dst + (size_t)p * ldd + dOff + k);
        if (accumulate) {
            float2 o = __bfloat1622float2(*d);
            v.x += o.x;
            v.y += o.y;
        }
        *d = __floats2bfloat162_rn(v.x, v.y);
    }
}

// The same element-wise layers over groups of 8 channels (one 16-byte load or
// store per group) with 32-bit indices: used when every channel count, leading
// dimension and offset is a multiple of 8, the pointers are 16-byte aligned
// and the element count fits 32 bits (the host checks); the arithmetic per
// channel is the one of the kernels above.
__device__ __forceinline__ void ld8(const __nv_bfloat16* p, float (&f)[8]) {
    const uint4 u = *reinterpret_cast<const uint4*>(p);
    const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float2 t = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w[k]));
        f[2 * k] = t.x;
        f[2 * k + 1] = t.y;
    }
}
__device__ __forceinline__ void st8(__nv_bfloat16* p, const float (&f)[8]) {
    uint32_t w[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        __nv_bfloat162 h2 = __floats2bfloat162_rn(f[2 * k], f[2 * k + 1]);
        w[k] = *reinterpret_cast<uint32_t*>(&h2);
    }
    *reinterpret_cast<uint4*>(p) = make_uint4(w[0], w[1], w[2], w[3]);
}

__global__ void k_relu_backward8(const __nv_bfloat16* out, uint32_t ldo, const __nv_bfloat16* dout, uint32_t ldd,
                                 __nv_bfloat16* dpre, uint32_t ldp, uint32_t groups, uint32_t total) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gstride()) {
        const uint32_t p = i / groups, k = (i - p * groups) * 8u;
        float o[8], d[8];
        ld8(out + (size_t)p * ldo + k, o);
        ld8(dout + (size_t)p * ldd + k, d);
#pragma unroll
        for (int j = 0; j < 8; ++j) d[j] = o[j] > 0.0f ? d[j] : 0.0f;
        st8(dpre + (size_t)p * ldp + k, d);
    }
}

__global__ void k_avgpool2_8(const __nv_bfloat16* in, uint32_t ldi, __nv_bfloat16* out, uint32_t ldo, uint32_t coOff,
                             uint32_t groups, uint32_t h, uint32_t w, uint32_t total) {
    pdlRelease();
    pdlWait();
    const uint32_t wo = w / 2u, ho = h / 2u;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gstride()) {
        const uint32_t q = i / groups, k = (i - q * groups) * 8u;
        const uint32_t x = q % wo, r = q / wo, y = r % ho, b = r / ho;
        const size_t base = ((size_t)(b * h + 2u * y) * w + 2u * x) * ldi + k;
        float s[8], t[8], u[8], v[8];
        ld8(in + base, s);
        ld8(in + base + ldi, t);
        ld8(in + base + (size_t)w * ldi, u);
        ld8(in + base + (size_t)w * ldi + ldi, v);
#pragma unroll
        for (int j = 0; j < 8; ++j) s[j] = 0.25f * (s[j] + t[j] + u[j] + v[j]);
        st8(out + (size_t)q * ldo + coOff + k, s);
    }
}

__global__ void k_avgpool2_backward8(const __nv_bfloat16* dout, uint32_t ldd, __nv_bfloat16* din, uint32_t ldi,
                                     uint32_t groups, uint32_t h, uint32_t w, int accumulate, uint32_t total) {
    // one thread per pooled pixel and group: its gradient goes to the 4 inputs
    const uint32_t wo = w / 2u, ho = h / 2u;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gstride()) {
        const uint32_t q = i / groups, k = (i - q * groups) * 8u;
        const uint32_t x = q % wo, r = q / wo, y = r % ho, b = r / ho;
        float d[8];
        ld8(dout + (size_t)q * ldd + k, d);
#pragma unroll
        for (int j = 0; j < 8; ++j) d[j] *= 0.25f;
        const size_t base = ((size_t)(b * h + 2u * y) * w + 2u * x) * ldi + k;
        const size_t offs[4] = {0, ldi, (size_t)w * ldi, (size_t)w * ldi + ldi};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            float v[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) v[j] = d[j];
            if (accumulate) {
                float o[8];
                ld8(din + base + offs[c], o);
#pragma unroll
                for (int j = 0; j < 8; ++j) v[j] += o[j];
            }
            st8(din + base + offs[c], v);
        }
    }
}

__global__ void k_upsample2_8(const __nv_bfloat16* in, uint32_t ldi, __nv_bfloat16* out, uint32_t ldo, uint32_t coOff,
                              uint32_t groups, uint32_t h, uint32_t w, uint32_t total) {
    // one thread per input pixel and group, written to its 2x2 outputs
    pdlRelease();
    pdlWait();
    const uint32_t W = 2u * w;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gstride()) {
        const uint32_t q = i / groups, k = (i - q * groups) * 8u;
        const uint32_t x = q % w, r = q / w, y = r % h, b = r / h;
        const uint4 v = *reinterpret_cast<const uint4*>(in + (size_t)q * ldi + k);
        const size_t o = ((size_t)(b * 2u * h + 2u * y) * W + 2u * x) * ldo + coOff + k;
        *reinterpret_cast<uint4*>(out + o) = v;
        *reinterpret_cast<uint4*>(out + o + ldo) = v;
        *reinterpret_cast<uint4*>(out + o + (size_t)W * ldo) = v;
        *reinterpret_cast<uint4*>(out + o + (size_t)W * ldo + ldo) = v;
    }
}

__global__ void k_upsample2_backward8(const __nv_bfloat16* dout, uint32_t ldd, uint32_t ciOff, __nv_bfloat16* din,
                                      uint32_t ldi, uint32_t groups, uint32_t h, uint32_t w, uint32_t total) {
    const uint32_t W = 2u * w;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gstride()) {
        const uint32_t q = i / groups, k = (i - q * groups) * 8u;
        const uint32_t x = q % w, r = q / w, y = r % h, b = r / h;
        const size_t base = ((size_t)(b * 2u * h + 2u * y) * W + 2u * x) * ldd + ciOff + k;
        float s[8], t[8], u[8], v[8];
        ld8(dout + base, s);
        ld8(dout + base + ldd, t);
        ld8(dout + base + (size_t)W * ldd, u);
        ld8(dout + base + (size_t)W * ldd + ldd, v);
#pragma unroll
        for (int j = 0; j < 8; ++j) s[j] = s[j] + t[j] + u[j] + v[j];
        st8(din + (size_t)q * ldi + k, s);
    }
}

__global__ void k_copy_channels8(const __nv_bfloat16* src, uint32_t lds, uint32_t sOff, __nv_bfloat16* dst,
                                 uint32_t ldd, uint32_t dOff, uint32_t groups, int accumulate, uint32_t total) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gstride()) {
        const uint32_t p = i / groups, k = (i - p * groups) * 8u;
        float v[8];
        ld8(src + (size_t)p * lds + sOff + k, v);
        __nv_bfloat16* d = dst + (size_t)p * ldd + dOff + k;
        if (accumulate) {
            float o[8];
            ld8(d, o);
#pragma unroll
            for (int j = 0; j < 8; ++j) v[j] += o[j];
        }
        st8(d, v);
    }
}

// Network input: 16 channels per pixel from the AOV planes (RGBA32F, image
// rows y0.., columns x0.. of a W_img-wide image; pixels outside the image are
// zero): log(1 + beauty) (3), albedo (3), normal in [-1, 1] (3), depth / (1 +
// depth) (1), zeros (6).
__global__ void k_pack_input(const float4* beauty, const float4* albedo, const float4* normal, const float4* depth,
                             uint32_t imgW, uint32_t imgH, uint32_t x0, uint32_t y0, __nv_bfloat16* out, uint32_t h,
                             uint32_t w, uint32_t batchIndex) {
    for (uint32_t i = gid(); i < h * w; i += gstride()) {
        uint32_t x = i % w, y = i / w;
        uint32_t ix = x0 + x, iy = y0 + y;
        float v[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) v[k] = 0.0f;
        if (ix < imgW && iy < imgH) {
            size_t s = (size_t)iy * imgW + ix;
            float4 b = beauty[s], a = albedo[s], nm = normal[s], d = depth[s];
            v[0] = log1pf(fmaxf(b.x, 0.0f));
            v[1] = log1pf(fmaxf(b.y, 0.0f));
            v[2] = log1pf(fmaxf(b.z, 0.0f));
            v[3] = a.x;
            v[4] = a.y;
            v[5] = a.z;
            v[6] = nm.x * 2.0f - 1.0f;
            v[7] = nm.y * 2.0f - 1.0f;
            v[8] = nm.z * 2.0f - 1.0f;
            float dd = fmaxf(d.x, 0.0f);
            v[9] = dd / (1.0f + dd);
        }
        __nv_bfloat16* o = out + ((size_t)batchIndex * h * w + i) * 16u;
#pragma unroll
        for (int k = 0; k < 16; k += 2)
            *reinterpret_cast<__nv_bfloat162*>(o + k) = __floats2bfloat162_rn(v[k], v[k + 1]);
    }
}

// L1 loss in log space against a target image (RGBA32F) and its gradient
// (scaled by 1 / (3 * pixels)) into the prediction's first 3 channels.  With
// `base` (the network input, whose first 3 channels are log(1 + noisy)), the
// prediction is a residual: the output is base + pred.
__global__ void k_l1_loss(const __nv_bfloat16* pred, uint32_t ldp, const __nv_bfloat16* base, uint32_t ldb,
                          const float4* target, uint32_t M, __nv_bfloat16* grad, uint32_t ldg, float* loss) {
    __shared__ float red[256];
    float s = 0.0f;
    const float scale = 1.0f / (3.0f * (float)M);
    for (uint32_t p = gid(); p < M; p += gstride()) {
        float4 t = target[p];
        float tl[3] = {log1pf(fmaxf(t.x, 0.0f)), log1pf(fmaxf(t.y, 0.0f)), log1pf(fmaxf(t.z, 0.0f))};
        float g[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float y = __bfloat162float(pred[(size_t)p * ldp + k]);
            if (base) y += __bfloat162float(base[(size_t)p * ldb + k]);
            float d = y - tl[k];
            s += fabsf(d);
            g[k] = (d > 0.0f ? scale : (d < 0.0f ? -scale : 0.0f));
        }
        __nv_bfloat16* gp = grad + (size_t)p * ldg;
        gp[0] = __float2bfloat16_rn(g[0]);
        gp[1] = __float2bfloat16_rn(g[1]);
        gp[2] = __float2bfloat16_rn(g[2]);
        for (uint32_t k = 3; k < ldg; ++k) gp[k] = __float2bfloat16_rn(0.0f);
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (uint32_t o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, red[0] * scale);
}

// Network output (log space, first 3 channels) to an RGBA32F image; alpha from
// `alphaSrc`.  With `base`: the output is base + pred (a residual over the
// network input's log(1 + noisy) channels), summed in FP32.
__global__ void k_unpack_output(const __nv_bfloat16* pred, uint32_t ldp, const __nv_bfloat16* base, uint32_t ldb,
                                uint32_t h, uint32_t w, const float4* alphaSrc, uint32_t imgW, uint32_t imgH,
                                uint32_t x0, uint32_t y0, float4* out) {
    for (uint32_t i = gid(); i < h * w; i += gstride()) {
        uint32_t ix = x0 + i % w, iy = y0 + i / w;
        if (ix >= imgW || iy >= imgH) continue;
        size_t s = (size_t)iy * imgW + ix;
        const __nv_bfloat16* p = pred + (size_t)i * ldp;
        float y[3] = {__bfloat162float(p[0]), __bfloat162float(p[1]), __bfloat162float(p[2])};
        if (base) {
            const __nv_bfloat16* b = base + (size_t)i * ldb;
            y[0] += __bfloat162float(b[0]);
            y[1] += __bfloat162float(b[1]);
            y[2] += __bfloat162float(b[2]);
        }
        out[s] = make_float4(fmaxf(expm1f(y[0]), 0.0f), fmaxf(expm1f(y[1]), 0.0f), fmaxf(expm1f(y[2]), 0.0f),
                             alphaSrc[s].w);
    }
}

// Adam on FP32 master weights; writes the bf16 forward weights and, for 3x3
// layers, the tap-flipped transposed copy the input gradient uses.
__global__ void k_adam(float* wts, const float* grad, float* m, float* v, uint32_t count, float lr, float b1, float b2,
                       float eps, float c1, float c2, __nv_bfloat16* wbf, __nv_bfloat16* wflip, uint32_t cout,
                       uint32_t cin) {
    for (uint32_t i = gid(); i < count; i += gstride()) {
        float g = grad[i];
        float mi = b1 * m[i] + (1.0f - b1) * g;
        float vi = b2 * v[i] + (1.0f - b2) * g * g;
        m[i] = mi;
        v[i] = vi;
        float wv = wts[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        wts[i] = wv;
        if (wbf) wbf[i] = __float2bfloat16_rn(wv);
        if (wflip) {
            uint32_t ci = i % cin, tap = (i / cin) % 9u, co = i / (9u * cin);
            wflip[((size_t)ci * 9u + (8u - tap)) * cout + co] = __float2bfloat16_rn(wv);
        }
    }
}

__global__ void k_weights_to_bf16(const float* wts, uint32_t count, __nv_bfloat16* wbf, __nv_bfloat16* wflip,
                                  uint32_t cout, uint32_t cin) {
    for (uint32_t i = gid(); i < count; i += gstride()) {
        float wv = wts[i];
        wbf[i] = __float2bfloat16_rn(wv);
        if (wflip) {
            uint32_t ci = i % cin, tap = (i / cin) % 9u, co = i / (9u * cin);
            wflip[((size_t)ci * 9u + (8u - tap)) * cout + co] = __float2bfloat16_rn(wv);
        }
    }
}

inline int gridFor(uint64_t work, int block = 256) {
    if (deviceProp().multiProcessorCount == 0) ensureDevice();
    uint64_t g = (work + block - 1) / block;
    uint64_t cap = (uint64_t)deviceProp().multiProcessorCount * 16u;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

inline bool aligned16(uint32_t v) { return v % 16u == 0u; }

// The 8-channel element-wise kernels apply: channel counts, leading
// dimensions and offsets multiples of 8, pointers 16-byte aligned, and the
// element count within 32 bits.
inline bool vec8(std::initializer_list<uint32_t> counts, std::initializer_list<const void*> ptrs, uint64_t total) {
    for (uint32_t v : counts)
        if (v % 8u) return false;
    for (const void* q : ptrs)
        if (reinterpret_cast<uintptr_t>(q) % 16u) return false;
    return total > 0 && total < (1ull << 31);
}

// 3: halo-row TMA + tcgen05 convolution where the layer fits it, else the
// per-tap one (default); 2: the per-tap persistent TMA + tcgen05 convolution;
// 1: the cp.async + tcgen05 one; 0: the mma.sync one.
int g_convPath = 3;

// Launch with programmatic stream serialization (see pdlWait); DK_PDL=0 launches
// plainly.
template <typename... KArgs, typename... Args>
cudaError_t launchPdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                      Args... args) {
    static int enabled = -1;
    if (enabled < 0) {
        const char* e = getenv("DK_PDL");
        enabled = (e && e[0] == '0') ? 0 : 1;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = enabled ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// dependency on libcuda).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encodeTiled() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

// Pipeline depth limit from the environment (a tuning knob, read at each
// launch), clamped to [lo, hi]; hi when unset.
uint32_t depthCap(const char* name, uint32_t lo, uint32_t hi) {
    const char* e = getenv(name);
    if (!e || !*e) return hi;
    const long v = strtol(e, nullptr, 10);
    return v < (long)lo ? lo : (v > (long)hi ? hi : (uint32_t)v);
}

// Output rows go through the epilogue's shared-memory transpose when the
// destination is overwritten and every pixel's channel run starts on a
// 16-byte boundary.
bool stagedStores(const ConvArgs& c) {
    return !c.accumulate && c.cout % 8u == 0u && c.ldo % 8u == 0u && c.coOff % 8u == 0u &&
           reinterpret_cast<uintptr_t>(c.out) % 16u == 0u;
}

// The halo-row kernel's launch, or kHaloUnfit (nothing launched) when the
// layer does not fit it: narrow images, or weights and halo ring beyond the
// shared memory of one CTA.
constexpr int kHaloUnfit = -1;
// `pool` (optional): where the 2x2 average of the output goes ([n][h / 2][w / 2]
// [poolLd]); *pooled says whether this launch writes it (tensor-store rows
// only), else the caller pools separately.
int launchConvHalo(const ConvArgs& c, cudaStream_t st, __nv_bfloat16* pool = nullptr, uint32_t poolLd = 0,
                   bool* pooled = nullptr) {
    if (pooled) *pooled = false;
    const uint32_t chunks = (c.cin + 63u) / 64u;
    const size_t optin = (size_t)deviceProp().sharedMemPerBlockOptin;
    // Vertical taps stacked into one MMA (N = 3 Cout <= 256) with a rolling
    // window of accumulator slots; DK_CONV_STACK=0 keeps one MMA per tap.
    const char* stackEnv = getenv("DK_CONV_STACK");
    const bool stack = c.cout * 3u <= 256u && !(stackEnv && stackEnv[0] == '0');
    // Stacked, a halo row is read only in its own step: two slots suffice
    // (one in use, one loading); else three rows are in use at a time.
    const uint32_t minRing = stack ? 2u : kHaloRingMin;
    if (c.w_ < 128u || c.cout > 256u || chunks > 2u || haloSmemBytes(c.cout, chunks, false, minRing, stack) > optin)
        return kHaloUnfit;
    const bool staged = stagedStores(c) && haloSmemBytes(c.cout, chunks, true, minRing, stack) <= optin;
    // Stacked layers of 16, 32 or 64 output channels write their rows with
    // TMA tensor stores (DK_CONV_TMA_STORE=0: through the lanes).
    const char* storeEnv = getenv("DK_CONV_TMA_STORE");
    const bool tmaStore = stack && staged && (c.cout == 16u || c.cout == 32u || c.cout == 64u) &&
                          !(storeEnv && storeEnv[0] == '0') &&
                          haloSmemBytes(c.cout, chunks, true, minRing, stack, true) <= optin;
    // The deepest ring that fits: every further slot is a row in flight.
    uint32_t ring = minRing;
    const uint32_t ringCap = depthCap("DK_CONV_HALO_RING", minRing, kHaloRingMax);
    while (ring < ringCap && haloSmemBytes(c.cout, chunks, staged, ring + 1u, stack, tmaStore) <= optin) ++ring;
    const size_t smem = haloSmemBytes(c.cout, chunks, staged, ring, stack, tmaStore);
    EncodeTiledFn enc = encodeTiled();
    if (!enc) return fail(DK_ERROR_COMMAND_FAILED, "cuTensorMapEncodeTiled is not available");
    HaloConvArgs a;
    a.bias = c.bias;
    a.out = c.out;
    a.n = c.n;
    a.h = c.h;
    a.w = c.w_;
    a.cin = c.cin;
    a.cout = c.cout;
    a.ldo = c.ldo;
    a.coOff = c.coOff;
    a.act = c.act;
    a.accumulate = c.accumulate;
    a.staged = staged ? 1 : 0;
    a.ring = ring;
    a.tmaStore = tmaStore ? 1u : 0u;
    a.slots = 0u;
    a.logSlots = 0u;
    if (stack) {
        a.slots = 1u;
        while (a.slots * 2u * c.cout <= 512u && a.slots * 2u <= kHaloAccMax) a.slots *= 2u;
        while ((1u << a.logSlots) < a.slots) ++a.logSlots;
    }
    // The pooled epilogue (DK_CONV_POOL=0: a separate pass): tensor-store rows,
    // slots in pairs of pairs, whole 2x2 windows, 16-byte pooled stores.
    const char* poolEnv = getenv("DK_CONV_POOL");
    const bool fusePool = pool && tmaStore && a.slots >= 4u && c.h % 2u == 0u && c.w_ % 2u == 0u && !c.accumulate &&
                          poolLd >= c.cout && poolLd % 8u == 0u && (reinterpret_cast<uintptr_t>(pool) & 15u) == 0u &&
                          !(poolEnv && poolEnv[0] == '0');
    a.pool = fusePool ? pool : nullptr;
    a.poolLd = fusePool ? poolLd : 0u;
    a.chunks = chunks;
    a.cols = 32u;
    while (a.cols < c.cout) a.cols <<= 1;
    a.tilesX = (c.w_ + 127u) / 128u;
    const uint32_t sms = (uint32_t)deviceProp().multiProcessorCount;
    const uint64_t rowsTotal = (uint64_t)c.n * a.tilesX * c.h;
    if (rowsTotal >= (1ull << 32)) return kHaloUnfit;
    a.totalRows = (uint32_t)rowsTotal;
    alignas(64) CUtensorMap mapIn, mapW;
    cuuint64_t dimIn[4] = {c.cin, c.w_, c.h, c.n};
    cuuint64_t strideIn[3] = {(cuuint64_t)c.ldi * 2u, (cuuint64_t)c.w_ * c.ldi * 2u, (cuuint64_t)c.h * c.w_ * c.ldi * 2u};
    cuuint32_t boxIn[4] = {64u, kHaloPix, 1u, 1u};
    cuuint32_t unit[4] = {1u, 1u, 1u, 1u};
    CUresult r = enc(&mapIn, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<__nv_bfloat16*>(c.in), dimIn, strideIn,
                     boxIn, unit, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(DK_ERROR_INVALID_ARGUMENT, "activation tensor map rejected");
    cuuint64_t dimW[3] = {c.cin, 9u, c.cout};
    cuuint64_t strideW[2] = {(cuuint64_t)c.cin * 2u, (cuuint64_t)9u * c.cin * 2u};
    cuuint32_t boxW[3] = {64u, 1u, c.cout};
    r = enc(&mapW, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<__nv_bfloat16*>(c.w), dimW, strideW, boxW, unit,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(DK_ERROR_INVALID_ARGUMENT, "weight tensor map rejected");
    // Output rows as boxes {Cout channels, 32 pixels} of the 4-D output (channels, x, y, image) at the
    // slice's channel offset; 2 Cout bytes per pixel row, swizzled like the staging boxes.
    alignas(64) CUtensorMap mapOut = mapIn;
    if (tmaStore) {
        cuuint64_t dimOut[4] = {c.ldo, c.w_, c.h, c.n};
        cuuint64_t strideOut[3] = {(cuuint64_t)c.ldo * 2u, (cuuint64_t)c.w_ * c.ldo * 2u,
                                   (cuuint64_t)c.h * c.w_ * c.ldo * 2u};
        cuuint32_t boxOut[4] = {c.cout, 32u, 1u, 1u};
        const CUtensorMapSwizzle swz = c.cout == 16u   ? CU_TENSOR_MAP_SWIZZLE_32B
                                       : c.cout == 32u ? CU_TENSOR_MAP_SWIZZLE_64B
                                                       : CU_TENSOR_MAP_SWIZZLE_128B;
        r = enc(&mapOut, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, c.out, dimOut, strideOut, boxOut, unit,
                CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return fail(DK_ERROR_INVALID_ARGUMENT, "output tensor map rejected");
    }
    using HaloKernel = void (*)(const CUtensorMap, const CUtensorMap, const CUtensorMap, HaloConvArgs);
    const uint32_t last = (c.cin - (chunks - 1u) * 64u + 15u) / 16u;
    HaloKernel kernels[2][2][4] = {
        {{k_conv3x3_halo<false, 1, 1>, k_conv3x3_halo<false, 1, 2>, k_conv3x3_halo<false, 1, 3>,
          k_conv3x3_halo<false, 1, 4>},
         {k_conv3x3_halo<false, 2, 1>, k_conv3x3_halo<false, 2, 2>, k_conv3x3_halo<false, 2, 3>,
          k_conv3x3_halo<false, 2, 4>}},
        {{k_conv3x3_halo<true, 1, 1>, k_conv3x3_halo<true, 1, 2>, k_conv3x3_halo<true, 1, 3>,
          k_conv3x3_halo<true, 1, 4>},
         {k_conv3x3_halo<true, 2, 1>, k_conv3x3_halo<true, 2, 2>, k_conv3x3_halo<true, 2, 3>,
          k_conv3x3_halo<true, 2, 4>}}};
    HaloKernel kernel = kernels[stack][chunks - 1u][last - 1u];
    static size_t configured[2][2][4] = {};
    if (smem > configured[stack][chunks - 1u][last - 1u]) {
        DK_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                "conv3x3 (halo) shared memory");
        configured[stack][chunks - 1u][last - 1u] = smem;
    }
    uint32_t grid = std::min(sms, a.totalRows);
    DK_CUDA(launchPdl(kernel, dim3(grid), dim3(320), smem, st, mapIn, mapW, mapOut, a), "conv3x3 (halo) launch");
    DK_CUDA(cudaGetLastError(), "conv3x3 (halo rows, TMA + tcgen05) launch");
    if (pooled) *pooled = fusePool;
    return DK_OK;
}

// rowTap: the row-tap mode (images at least 128 pixels wide); else one stage
// per (tap, chunk) over 2-D tiles.
int launchConvTma(const ConvArgs& c, cudaStream_t st, bool rowTap) {
    rowTap = rowTap && c.w_ >= 128u;
    EncodeTiledFn enc = encodeTiled();
    if (!enc) return fail(DK_ERROR_COMMAND_FAILED, "cuTensorMapEncodeTiled is not available");
    TmaConvArgs a;
    a.bias = c.bias;
    a.out = c.out;
    a.n = c.n;
    a.h = c.h;
    a.w = c.w_;
    a.cin = c.cin;
    a.cout = c.cout;
    a.ldo = c.ldo;
    a.coOff = c.coOff;
    a.act = c.act;
    a.accumulate = c.accumulate;
    uint32_t tw = 1;
    while (tw * 2u <= c.w_ && tw < 128u) tw *= 2u;
    if (rowTap) tw = 128u;
    a.tw = tw;
    a.th = 128u / tw;
    a.tilesX = (c.w_ + a.tw - 1) / a.tw;
    a.tilesY = (c.h + a.th - 1) / a.th;
    a.numTiles = a.tilesX * a.tilesY * c.n;
    a.chunks = (c.cin + 63u) / 64u;
    a.cols = 32u;
    while (a.cols < c.cout) a.cols <<= 1;
    alignas(64) CUtensorMap mapIn, mapW;
    cuuint64_t dimIn[4] = {c.cin, c.w_, c.h, c.n};
    cuuint64_t strideIn[3] = {(cuuint64_t)c.ldi * 2u, (cuuint64_t)c.w_ * c.ldi * 2u, (cuuint64_t)c.h * c.w_ * c.ldi * 2u};
    cuuint32_t boxIn[4] = {64u, rowTap ? kHaloPix : a.tw, a.th, 1u};
    cuuint32_t unit[4] = {1u, 1u, 1u, 1u};
    CUresult r = enc(&mapIn, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<__nv_bfloat16*>(c.in), dimIn, strideIn,
                     boxIn, unit, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(DK_ERROR_INVALID_ARGUMENT, "activation tensor map rejected");
    cuuint64_t dimW[3] = {c.cin, 9u, c.cout};
    cuuint64_t strideW[2] = {(cuuint64_t)c.cin * 2u, (cuuint64_t)9u * c.cin * 2u};
    cuuint32_t boxW[3] = {64u, 1u, c.cout};
    r = enc(&mapW, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<__nv_bfloat16*>(c.w), dimW, strideW, boxW, unit,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(DK_ERROR_INVALID_ARGUMENT, "weight tensor map rejected");
    const size_t optin = (size_t)deviceProp().sharedMemPerBlockOptin;
    const uint32_t minStages = rowTap ? 2u : kTmaStagesMin;
    if (tmaSmemBytes(c.cout, false, minStages, rowTap) > optin) {
        if (rowTap) return launchConvTma(c, st, false);
        return fail(DK_ERROR_INVALID_ARGUMENT, "conv3x3: the layer does not fit shared memory");
    }
    const bool staged = stagedStores(c) && tmaSmemBytes(c.cout, true, minStages, rowTap) <= optin;
    uint32_t stages = minStages;
    const uint32_t stageCap = depthCap("DK_CONV_STAGES", minStages, kTmaStagesMax);
    while (stages < stageCap && tmaSmemBytes(c.cout, staged, stages + 1u, rowTap) <= optin) ++stages;
    a.staged = staged ? 1 : 0;
    a.stages = stages;
    size_t smem = tmaSmemBytes(c.cout, staged, stages, rowTap);
    static size_t configured[2] = {0, 0};
    if (smem > configured[rowTap]) {
        DK_CUDA(cudaFuncSetAttribute(rowTap ? k_conv3x3_tma<true> : k_conv3x3_tma<false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                "conv3x3 shared memory");
        configured[rowTap] = smem;
    }
    uint32_t grid = (uint32_t)deviceProp().multiProcessorCount;
    if (grid > a.numTiles) grid = a.numTiles;
    if (rowTap)
        DK_CUDA(launchPdl(k_conv3x3_tma<true>, dim3(grid), dim3(320), smem, st, mapIn, mapW, a), "conv3x3 launch");
    else
        DK_CUDA(launchPdl(k_conv3x3_tma<false>, dim3(grid), dim3(320), smem, st, mapIn, mapW, a), "conv3x3 launch");
    DK_CUDA(cudaGetLastError(), "conv3x3 (TMA + tcgen05) launch");
    return DK_OK;
}

}  // namespace
}  // namespace dk

using bf16 = __nv_bfloat16;

extern "C" {

int dk_unet_conv3x3(const void* in, uint32_t n, uint32_t h, uint32_t w, uint32_t cin, uint32_t ldi,
                    const void* weight, const float* bias, uint32_t cout, void* out, uint32_t ldo, uint32_t coOff,
                    int act, int accumulate, void* stream) {
    if (!in || !weight || !out) return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_unet_conv3x3: null argument");
    if (!dk::aligned16(cin) || !dk::aligned16(cout) || ldi < cin || ldo < coOff + cout || ldi % 8u || ldo % 2u ||
        coOff % 2u)
        return dk::fail(DK_ERROR_INVALID_ARGUMENT,
                        "dk_unet_conv3x3: channel counts must be multiples of 16 within their leading dimensions");
    uint64_t M = (uint64_t)n * h * w;
    if (M == 0) return DK_OK;
    if (M >= (1ull << 31)) return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_unet_conv3x3: tensor too large");
    dk::ConvArgs a{static_cast<const bf16*>(in), static_cast<const bf16*>(weight), bias, static_cast<bf16*>(out),
                   n, h, w, cin, ldi, cout, ldo, coOff, (uint32_t)M, act, accumulate};
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (dk::g_convPath == 3 && cout <= 256u) {
        int rc = dk::launchConvHalo(a, st);
        if (rc != dk::kHaloUnfit) return rc;
    }
    if (dk::g_convPath >= 2 && cout <= 256u) {
        int rc = dk::launchConvTma(a, st, dk::g_convPath == 3);
        if (rc != DK_OK) return rc;
        return DK_OK;
    }
    if (dk::g_convPath == 1 && cout <= 256u) {
        uint32_t cols = 32u;
        while (cols < cout) cols <<= 1;
        size_t smem = dk::tcSmemBytes(cout);
        static size_t configured = 0;
        if (smem > configured) {
            DK_CUDA(cudaFuncSetAttribute(dk::k_conv3x3_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                    "conv3x3 shared memory");
            configured = smem;
        }
        dk::k_conv3x3_tc<<<(uint32_t)((M + dk::kTcRows - 1) / dk::kTcRows), 128, smem, st>>>(a, cols);
        DK_CUDA(cudaGetLastError(), "conv3x3 (tcgen05) launch");
        return DK_OK;
    }
    dim3 grid((uint32_t)((M + dk::kBM - 1) / dk::kBM), 1);
    if (cout % 64u == 0) {
        grid.y = cout / 64u;
        dk::k_conv3x3_fwd<64><<<grid, 128, 0, st>>>(a);
    } else if (cout % 32u == 0) {
        grid.y = cout / 32u;
        dk::k_conv3x3_fwd<32><<<grid, 128, 0, st>>>(a);
    } else {
        grid.y = cout / 16u;
        dk::k_conv3x3_fwd<16><<<grid, 128, 0, st>>>(a);
    }
    DK_CUDA(cudaGetLastError(), "conv3x3 launch");
    return DK_OK;
}

int dk_unet_conv3x3_wgrad(const void* in, uint32_t ldi, const void* dout, uint32_t ldd, uint32_t n, uint32_t h,
                          uint32_t w, uint32_t cin, uint32_t cout, float* dweight, void* stream) {
    if (!in || !dout || !dweight) return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_unet_conv3x3_wgrad: null argument");
    if (!dk::aligned16(cin) || !dk::aligned16(cout) || ldi < cin || ldd < cout || ldi % 8u || ldd % 8u)
        return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_unet_conv3x3_wgrad: channel counts must be multiples of 16");
    uint64_t M = (uint64_t)n * h * w;
    if (M == 0) return DK_OK;
    if (M >= (1ull << 31)) return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_unet_conv3x3_wgrad: tensor too large");
    uint32_t tiles = ((cout + 63u) / 64u) * ((cin + 63u) / 64u);
    // Enough pixel chunks to fill the GPU several times over, 32-pixel aligned.
    if (dk::deviceProp().multiProcessorCount == 0) dk::ensureDevice();
    uint64_t target = (uint64_t)dk::deviceProp().multiProcessorCount * 8u;
    uint64_t perTile = (target + 9u * tiles - 1) / (9u * tiles);
    uint64_t chunk = (M + perTile - 1) / perTile;
    chunk = ((chunk + 31u) / 32u) * 32u;
    if (chunk < 256u) chunk = 256u;
    dk::WgradArgs a{static_cast<const bf16*>(in), static_cast<const bf16*>(dout), dweight, n, h, w, cin, ldi, cout,
                    ldd, (uint32_t)M, (uint32_t)chunk};
    dim3 grid((uint32_t)((M + chunk - 1) / chunk), tiles, 9);
    dk::k_conv3x3_wgrad<<<grid, 128, 0, static_cast<cudaStream_t>(stream)>>>(a);
    DK_CUDA(cudaGetLastError(), "conv3x3 wgrad launch");
    return DK_OK;
}

int dk_unet_relu_backward(const void* out, uint32_t ldo, const void* dout, uint32_t ldd, void* dpre, uint32_t ldp,
                          uint32_t c, uint32_t pixels, void* stream) {
    if (!out || !dout || !dpre || c % 2u) return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_unet_relu_backward");
    const uint64_t total8 = (uint64_t)pixels * (c / 8u);
    if (dk::vec8({c, ldo, ldd, ldp}, {out, dout, dpre}, total8)) {
        dk::k_relu_backward8<<<dk::gridFor(total8), 256, 0, static_cast<cudaStream_t>(stream)>>>(
            static_cast<const bf16*>(out), ldo, static_cast<const bf16*>(dout), ldd, static_cast<bf16*>(dpre), ldp,
            c / 8u, (uint32_t)total8);
        DK_CUDA(cudaGetLastError(), "relu backward launch");
        return DK_OK;
    }
    dk::k_relu_backward<<<dk::gridFor((uint64_t)pixels * c / 2), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const bf16*>(out), ldo, static_cast<const bf16*>(dout), ldd, static_cast<bf16*>(dpre), ldp, c,
        pixels);
    DK_CUDA(cudaGetLastError(), "relu backward launch");
    return DK_OK;
}

int dk_unet_bias_grad(const void* dpre, uint32_t ld, uint32_t c, uint32_t pixels, float* dbias, void* stream) {
    if (!dpre || !dbias || c == 0 || c > 256u) return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_unet_bias_grad");
    uint32_t lanes = 256u / c;
    uint64_t blocks = ((uint64_t)pixels + lanes * 64u - 1) / (lanes * 64u);
    int grid = (int)(blocks < 1 ? 1 : (blocks > 1024 ? 1024 : blocks));
    dk::k_bias_grad<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<const bf16*>(dpre), ld, c, pixels,
                                                                          dbias);
    DK_CUDA(cudaGetLastError(), "bias grad launch");
    return DK_OK;
}

int dk_unet_avgpool2(const void* in, uint32_t ldi, void* out, uint32_t ldo, uint32_t coOff, uint32_t c, uint32_t n,
                     uint32_t h, uint32_t w, void* stream) {
    if (!in || !out || c % 2u || h % 2u || w % 2u) return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_unet_avgpool2");
    const uint64_t total8 = (uint64_t)n * (h / 2u) * (w / 2u) * (c / 8u);
    if (dk::vec8({c, ldi, ldo, coOff}, {in, out}, total8)) {
        DK_CUDA(dk::launchPdl(dk::k_avgpool2_8, dim3(dk::gridFor(total8)), dim3(256), 0,
                              static_cast<cudaStream_t>(stream), static_cast<const bf16*>(in), ldi,
                              static_cast<bf16*>(out), ldo, coOff, c / 8u, h, w, (uint32_t)total8),
                "avgpool launch");
        return DK_OK;
    }
    dk::k_avgpool2<<<dk::gridFor((uint64_t)n * h * w / 4 * c / 2), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const bf16*>(in), ldi, static_cast<bf16*>(out), ldo, coOff, c, n, h, w);
    DK_CUDA(cudaGetLastError(), "avgpool launch");
    return DK_OK;
}

int dk_unet_conv3x3_avgpool2(const void* in, uint32_t n, uint32_t h, uint32_t w, uint32_t cin, uint32_t ldi,
                             const void* weight, const float* bias, uint32_t cout, void* out, uint32_t ldo,
                             uint32_t coOff, int act, void* pool, uint32_t poolLd, void* stream) {
    if (!pool || h % 2u || w % 2u || poolLd < cout)
        return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_unet_conv3x3_avgpool2: pool target or odd extent");
    if (dk::g_convPath == 3 && cout <= 256u && in && weight && out && dk::aligned16(cin) && dk::aligned16(cout) &&
        ldi >= cin && ldo >= coOff + cout && ldi % 8u == 0u && ldo % 2u == 0u && coOff % 2u == 0u &&
        (uint64_t)n * h * w > 0 && (uint64_t)n * h * w < (1ull << 31)) {
        dk::ConvArgs a{static_cast<const bf16*>(in), static_cast<const bf16*>(weight), bias, static_cast<bf16*>(out),
                       n, h, w, cin, ldi, cout, ldo, coOff, (uint32_t)((uint64_t)n * h * w), act, 0};
        bool pooled = false;
        int rc = dk::launchConvHalo(a, static_cast<cudaStream_t>(stream), static_cast<bf16*>(pool), poolLd, &pooled);
        if (rc != dk::kHaloUnfit) {
            if (rc != DK_OK || pooled) return rc;
            return dk_unet_avgpool2(static_cast<const bf16*>(out) + coOff, ldo, pool, poolLd, 0u, cout, n, h, w, stream);
        }
    }
    int rc = dk_unet_conv3x3(in, n, h, w, cin, ldi, weight, bias, cout, out, ldo, coOff, act, 0, stream);
    if (rc != DK_OK) return rc;
    return dk_unet_avgpool2(static_cast<const bf16*>(out) + coOff, ldo, pool, poolLd, 0u, cout, n, h, w, stream);
}

int dk_unet_avgpool2_backward(const void* dout, uint32_t ldd, void* din, uint32_t ldi, uint32_t c, uint32_t n,
                              uint32_t h, uint32_t w, int accumulate, void* stream) {
    if (!dout || !din || c % 2u || h % 2u || w % 2u)
        return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_unet_avgpool2_backward");
    const uint64_t total8 = (uint64_t)n * (h / 2u) * (w / 2u) * (c / 8u);
    if (dk::vec8({c, ldd, ldi}, {dout, din}, total8)) {
        dk::k_avgpool2_backward8<<<dk::gridFor(total8), 256, 0, static_cast<cudaStream_t>(stream)>>>(
            static_cast<const bf16*>(dout), ldd, static_cast<bf16*>(din), ldi, c / 8u, h, w, accumulate,
            (uint32_t)total8);
        DK_CUDA(cudaGetLastError(), "avgpool backward launch");
        return DK_OK;
    }
    dk::k_avgpool2_backward<<<dk::gridFor((uint64_t)n * h * w * c / 2), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const bf16*>(dout), ldd, static_cast<bf16*>(din), ldi, c, n, h, w, accumulate);
    DK_CUDA(cudaGetLastError(), "avgpool backward launch");
    return DK_OK;
}

int dk_unet_upsample2(const void* in, uint32_t ldi, void* out, uint32_t ldo, uint32_t coOff, uint32_t c, uint32_t n,
                      uint32_t h, uint32_t w, void* stream) {
    if (!in || !out || c % 2u) return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_unet_upsample2");
    const uint64_t total8 = (uint64_t)n * h * w * (c / 8u);
    if (dk::vec8({c, ldi, ldo, coOff}, {in, out}, total8)) {
        DK_CUDA(dk::launchPdl(dk::k_upsample2_8, dim3(dk::gridFor(total8)), dim3(256), 0,
                              static_cast<cudaStream_t>(stream), static_cast<const bf16*>(in), ldi,
                              static_cast<bf16*>(out), ldo, coOff, c / 8u, h, w, (uint32_t)total8),
                "upsample launch");
        return DK_OK;
    }
    dk::k_upsample2<<<dk::gridFor((uint64_t)n * h * w * 4 * c / 2), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const bf16*>(in), ldi, static_cast<bf16*>(out), ldo, coOff, c, n, h, w);
    DK_CUDA(cudaGetLastError(), "upsample launch");
    return DK_OK;
}

int dk_unet_upsample2_backward(const void* dout, uint32_t ldd, uint32_t ciOff, void* din, uint32_t ldi, uint32_t c,
                               uint32_t n, uint32_t h, uint32_t w, void* stream) {
    if (!dout || !din || c % 2u) return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_unet_upsample2_backward");
    const uint64_t total8 = (uint64_t)n * h * w * (c / 8u);
    if (dk::vec8({c, ldd, ciOff, ldi}, {dout, din}, total8)) {
        dk::k_upsample2_backward8<<<dk::gridFor(total8), 256, 0, static_cast<cudaStream_t>(stream)>>>(
            static_cast<const bf16*>(dout), ldd, ciOff, static_cast<bf16*>(din), ldi, c / 8u, h, w, (uint32_t)total8);
        DK_CUDA(cudaGetLastError(), "upsample backward launch");
        return DK_OK;
    }
    dk::k_upsample2_backward<<<dk::gridFor((uint64_t)n * h * w * c / 2), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const bf16*>(dout), ldd, ciOff, static_cast<bf16*>(din), ldi, c, n, h, w);
    DK_CUDA(cudaGetLastError(), "upsample backward launch");
    return DK_OK;
}

int dk_unet_copy_channels(const void* src, uint32_t lds, uint32_t sOff, void* dst, uint32_t ldd, uint32_t dOff,
                          uint32_t c, uint32_t pixels, int accumulate, void* stream) {
    if (!src || !dst || c % 2u || sOff % 2u || dOff % 2u)
        return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_unet_copy_channels");
    const uint64_t total8 = (uint64_t)pixels * (c / 8u);
    if (dk::vec8({c, lds, sOff, ldd, dOff}, {src, dst}, total8)) {
        dk::k_copy_channels8<<<dk::gridFor(total8), 256, 0, static_cast<cudaStream_t>(stream)>>>(
            static_cast<const bf16*>(src), lds, sOff, static_cast<bf16*>(dst), ldd, dOff, c / 8u, accumulate,
            (uint32_t)total8);
        DK_CUDA(cudaGetLastError(), "copy channels launch");
        return DK_OK;
    }
    dk::k_copy_channels<<<dk::gridFor((uint64_t)pixels * c / 2), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const bf16*>(src), lds, sOff, static_cast<bf16*>(dst), ldd, dOff, c, pixels, accumulate);
    DK_CUDA(cudaGetLastError(), "copy channels launch");
    return DK_OK;
}

int dk_unet_pack_input(const float* beauty, const float* albedo, const float* normal, const float* depth,
                       uint32_t imgW, uint32_t imgH, uint32_t x0, uint32_t y0, void* out, uint32_t h, uint32_t w,
                       uint32_t batchIndex, void* stream) {
    if (!beauty || !albedo || !normal || !depth || !out) return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_unet_pack_input");
    dk::k_pack_input<<<dk::gridFor((uint64_t)h * w), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<const float4*>(beauty), reinterpret_cast<const float4*>(albedo),
        reinterpret_cast<const float4*>(normal), reinterpret_cast<const float4*>(depth), imgW, imgH, x0, y0,
        static_cast<bf16*>(out), h, w, batchIndex);
    DK_CUDA(cudaGetLastError(), "pack input launch");
    return DK_OK;
}

int dk_unet_l1_loss(const void* pred, uint32_t ldp, const float* target, uint32_t pixels, void* grad, uint32_t ldg,
                    float* loss, void* stream) {
    if (!pred || !target || !grad || !loss || ldp < 3u || ldg < 3u)
        return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_unet_l1_loss");
    dk::k_l1_loss<<<dk::gridFor(pixels), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const bf16*>(pred), ldp, nullptr, 0u, reinterpret_cast<const float4*>(target), pixels,
        static_cast<bf16*>(grad), ldg, loss);
    DK_CUDA(cudaGetLastError(), "loss launch");
    return DK_OK;
}

int dk_unet_l1_loss_residual(const void* pred, uint32_t ldp, const void* base, uint32_t ldb, const float* target,
                             uint32_t pixels, void* grad, uint32_t ldg, float* loss, void* stream) {
    if (!pred || !base || !target || !grad || !loss || ldp < 3u || ldb < 3u || ldg < 3u)
        return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_unet_l1_loss_residual");
    dk::k_l1_loss<<<dk::gridFor(pixels), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const bf16*>(pred), ldp, static_cast<const bf16*>(base), ldb,
        reinterpret_cast<const float4*>(target), pixels, static_cast<bf16*>(grad), ldg, loss);
    DK_CUDA(cudaGetLastError(), "loss launch");
    return DK_OK;
}

int dk_unet_unpack_output(const void* pred, uint32_t ldp, uint32_t h, uint32_t w, const float* alphaSrc, uint32_t imgW,
                          uint32_t imgH, uint32_t x0, uint32_t y0, float* out, void* stream) {
    if (!pred || !alphaSrc || !out) return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_unet_unpack_output");
    dk::k_unpack_output<<<dk::gridFor((uint64_t)h * w), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const bf16*>(pred), ldp, nullptr, 0u, h, w, reinterpret_cast<const float4*>(alphaSrc), imgW, imgH,
        x0, y0, reinterpret_cast<float4*>(out));
    DK_CUDA(cudaGetLastError(), "unpack output launch");
    return DK_OK;
}

int dk_unet_unpack_output_residual(const void* pred, uint32_t ldp, const void* base, uint32_t ldb, uint32_t h,
                                   uint32_t w, const float* alphaSrc, uint32_t imgW, uint32_t imgH, uint32_t x0,
                                   uint32_t y0, float* out, void* stream) {
    if (!pred || !base || !alphaSrc || !out || ldb < 3u)
        return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_unet_unpack_output_residual");
    dk::k_unpack_output<<<dk::gridFor((uint64_t)h * w), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const bf16*>(pred), ldp, static_cast<const bf16*>(base), ldb, h, w,
        reinterpret_cast<const float4*>(alphaSrc), imgW, imgH, x0, y0, reinterpret_cast<float4*>(out));
    DK_CUDA(cudaGetLastError(), "unpack output launch");
    return DK_OK;
}

int dk_unet_adam(float* weights, const float* grad, float* m, float* v, uint32_t count, float lr, float beta1,
                 float beta2, float eps, uint32_t step, void* wbf16, void* wflip, uint32_t cout, uint32_t cin,
                 void* stream) {
    if (!weights || !grad || !m || !v || step == 0) return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_unet_adam");
    float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    dk::k_adam<<<dk::gridFor(count), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        weights, grad, m, v, count, lr, beta1, beta2, eps, c1, c2, static_cast<bf16*>(wbf16), static_cast<bf16*>(wflip),
        cout, cin);
    DK_CUDA(cudaGetLastError(), "adam launch");
    return DK_OK;
}

int dk_unet_set_conv_path(int path) {
    if (path < 0 || path > 3) return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_unet_set_conv_path: 0, 1, 2 or 3");
    dk::g_convPath = path;
    return DK_OK;
}

int dk_unet_error(int* out) {
    if (!out) return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_unet_error: null argument");
    int zero = 0;
    DK_CUDA(cudaMemcpyFromSymbol(out, dk::g_unetError, sizeof(int)), "read denoiser error flag");
    DK_CUDA(cudaMemcpyToSymbol(dk::g_unetError, &zero, sizeof(int)), "clear denoiser error flag");
    return DK_OK;
}

int dk_unet_weights_to_bf16(const float* weights, uint32_t count, void* wbf16, void* wflip, uint32_t cout, uint32_t cin,
                            void* stream) {
    if (!weights || !wbf16) return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_unet_weights_to_bf16");
    dk::k_weights_to_bf16<<<dk::gridFor(count), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        weights, count, static_cast<bf16*>(wbf16), static_cast<bf16*>(wflip), cout, cin);
    DK_CUDA(cudaGetLastError(), "weights launch");
    return DK_OK;
}

}  // extern "C"
