// Learned warm start for newly created contacts (no counterpart in the reference, whose
// new contacts start from zero impulse, Contact.cs:727).
//
// Network: 24 features -> 64 -> 64 -> 3 (normal, tangent-1, tangent-2 impulse), ReLU,
// BF16 weights and activations, FP32 accumulation and biases.  Every GEMM of the
// forward and backward pass runs on the 5th-generation tensor cores: operands are staged
// by the CTA's threads into shared memory in the K-major core-matrix layout (8 rows x
// 16 bytes per core matrix, no swizzle), one elected thread issues tcgen05.mma with the
// FP32 accumulator in tensor memory, tcgen05.commit signals an mbarrier, and the four
// warps read their 32 accumulator lanes back with tcgen05.ld for the epilogue (bias,
// ReLU, BF16 rounding, masks, gradient atomics).  One CTA handles 128 samples at a time
// (M = 128, one TMEM lane per sample).
//
// Features of a new contact (all world frame): normal (3), tangent 1 (3), relative
// velocity along n, t1, t2 (3), penetration depth (1), inverse masses (2), diagonals of
// both world inverse inertias (6), both lever arms (6).
#include "jg_world.cuh"
#include <cuda_bf16.h>
#include <vector>
#include <string>
#include <cstring>
#include <cmath>
#include <algorithm>

struct jg_world;
void jg_world_invalidate_graphs(jg_world* w);
WorldDev& jg_world_dev(jg_world* w);
cudaStream_t jg_world_stream(jg_world* w);
int jg_world_nsm(jg_world* w);
void jg_world_set_mlp_ready(jg_world* w, bool r);
void*& jg_world_mlp(jg_world* w);
int* jg_world_dst_index(jg_world* w);
void jg_set_error(const char* msg);

namespace {

constexpr int IN = 24, K1 = 32, HID = 64, OUT = 3, N3 = 16, TILE = 128;
// float parameter layout (jg_mlp_load / jg_mlp_export); gradients use the first NW
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + HID * IN, OFF_W2 = OFF_B1 + HID, OFF_B2 = OFF_W2 + HID * HID,
              OFF_W3 = OFF_B2 + HID, OFF_B3 = OFF_W3 + OUT * HID, NW = OFF_B3 + OUT;
constexpr int OFF_MEAN = NW, OFF_SCALE = OFF_MEAN + IN, OFF_OSCALE = OFF_SCALE + IN, NPARAM = OFF_OSCALE + OUT;
// BF16 operand copies (row-major, B operands "N rows x K"): W1 [64][32], W2 [64][64],
// W3 [16][64] (rows 3.. zero), W3t [64][16] (W3 transposed, cols 3.. zero), W2t [64][64]
constexpr int WB_W1 = 0, WB_W2 = WB_W1 + HID * K1, WB_W3 = WB_W2 + HID * HID, WB_W3T = WB_W3 + N3 * HID,
              WB_W2T = WB_W3T + HID * N3, WB_TOTAL = WB_W2T + HID * HID;
// shared memory regions (bytes), all 1024-aligned
constexpr int S_X = 0, S_W1 = S_X + TILE * K1 * 2, S_H1 = S_W1 + HID * K1 * 2, S_W2 = S_H1 + TILE * HID * 2,
              S_H2 = S_W2 + HID * HID * 2, S_W3 = S_H2 + TILE * HID * 2, S_FWD_END = S_W3 + N3 * HID * 2;
constexpr int S_DY = S_FWD_END, S_W3T = S_DY + TILE * N3 * 2, S_DZ2 = S_W3T + HID * N3 * 2,
              S_W2T = S_DZ2 + TILE * HID * 2, S_A = S_W2T + HID * HID * 2, S_B = S_A + TILE * TILE * 2,
              S_TRAIN_END = S_B + 96 * TILE * 2;
constexpr int TMEM_COLS = 128;

struct MlpArgs {
    const __nv_bfloat16* wb;
    const float* p;        // FP32 parameters (biases and normalisation read here)
    const float* X;        // [n][24] raw features
    const float* T;        // [n][3] targets (training)
    const int* nptr;       // device count (warm start) or null
    int n;
    float* out;            // [n][3] predictions (de-normalised)
    float* grad;           // [NW]
    float* loss;           // [1] sum of squared errors
    int* status;
};

// ---- PTX wrappers ------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned long long gtime() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// byte offset of element (r, k) of a K-major tile with K columns (core matrices of 8 x 16 B)
__device__ __forceinline__ int km_off(int r, int k, int K) {
    return (((r >> 3) * (K >> 3) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1);
}
// shared memory matrix descriptor: K-major, no swizzle; LBO = next core matrix along K
// (128 B), SBO = next group of 8 rows (K/8 core matrices), descriptor version 1
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, int K) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)(128 >> 4) << 16;
    d |= (uint64_t)(((K >> 3) * 128) >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}
// instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both K-major
__device__ __forceinline__ uint32_t instr_desc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, int acc) {
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
                 :: "r"(tmem_d), "l"(a), "l"(b), "r"(idesc), "r"(acc) : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(mbar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// bounded wait for an mbarrier phase: false after about a second
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase) {
    unsigned long long t0 = gtime();
    for (;;) {
        uint32_t ok;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(ok) : "r"(mbar), "r"(phase) : "memory");
        if (ok) return true;
        if (gtime() - t0 > 1000000000ull) return false;
    }
}
// 16 consecutive FP32 accumulator columns of this warp's 32 lanes
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// Stages a row-major BF16 matrix [rows][K] into the K-major core-matrix layout.
__device__ __forceinline__ void stage_rows(unsigned char* dst, const __nv_bfloat16* src, int rows, int K) {
    const int chunks = rows * (K >> 3);
    for (int c = threadIdx.x; c < chunks; c += blockDim.x) {
        int r = c / (K >> 3), k8 = c - r * (K >> 3);
        *(uint4*)(dst + km_off(r, k8 * 8, K)) = *(const uint4*)(src + (size_t)r * K + k8 * 8);
    }
}
__device__ __forceinline__ void put_bf16(unsigned char* base, int off, float v) {
    *(__nv_bfloat16*)(base + off) = __float2bfloat16_rn(v);
}
__device__ __forceinline__ float get_bf16(const unsigned char* base, int off) {
    return __bfloat162float(*(const __nv_bfloat16*)(base + off));
}

// Issues a GEMM D[128 x N] (tmem column col) = A[128 x K] * B[N x K]^T from shared memory.
__device__ __forceinline__ void gemm(uint32_t tmem, int col, uint32_t a, uint32_t b, int N, int K, uint32_t mbar) {
    const uint32_t idesc = instr_desc(128, N);
    for (int ks = 0; ks < K / 16; ks++)
        mma_bf16(tmem + col, smem_desc(a + ks * 256, K), smem_desc(b + ks * 256, K), idesc, ks > 0 ? 1 : 0);
    mma_commit(mbar);
}

// All threads: make the staged operands visible to the tensor core, run one GEMM, wait.
__device__ __forceinline__ bool run_gemm(uint32_t tmem, int col, uint32_t a, uint32_t b, int N, int K, uint32_t mbar,
                                         uint32_t& phase, int* abort_flag) {
    proxy_fence();
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0) {
        tc_fence_after();
        gemm(tmem, col, a, b, N, K, mbar);
    }
    bool ok = mbar_wait(mbar, phase);
    phase ^= 1u;
    // every thread takes the same branch, so warp-collective tensor-memory loads stay converged
    const int failed = __syncthreads_or(!ok);
    tc_fence_after();
    if (failed) {
        if (threadIdx.x == 0) *abort_flag = 1;
        return false;
    }
    return true;
}

struct Ctx {
    unsigned char* s;
    uint32_t sbase, tmem, mbar;
    uint32_t phase;
    int* abort_flag;
};

// Forward pass of one tile of rows [r0, r0 + 128): leaves H1, H2 (BF16) in shared memory
// and returns this thread's normalised outputs y[3] (row threadIdx.x).
__device__ bool forward_tile(Ctx& c, const MlpArgs& g, int r0, int n, float* y, float* xrow) {
    const int r = threadIdx.x, warp = r >> 5;
    const float* p = g.p;
    // features -> normalised BF16 row (K padded to 32)
    float x[K1];
#pragma unroll
    for (int f = 0; f < K1; f++) x[f] = 0.f;
    if (r0 + r < n) {
#pragma unroll
        for (int f = 0; f < IN; f++) x[f] = (g.X[(size_t)(r0 + r) * IN + f] - p[OFF_MEAN + f]) * p[OFF_SCALE + f];
    }
#pragma unroll
    for (int f = 0; f < K1; f++) {
        x[f] = __bfloat162float(__float2bfloat16_rn(x[f]));
        put_bf16(c.s + S_X, km_off(r, f, K1), x[f]);
        if (xrow) xrow[f] = x[f];
    }
    const uint32_t lane_addr = c.tmem + ((uint32_t)(32 * warp) << 16);
    // layer 1
    if (!run_gemm(c.tmem, 0, c.sbase + S_X, c.sbase + S_W1, HID, K1, c.mbar, c.phase, c.abort_flag)) return false;
    for (int q = 0; q < HID / 16; q++) {
        float v[16];
        tmem_ld16(lane_addr + 16 * q, v);
#pragma unroll
        for (int i = 0; i < 16; i++) {
            int j = 16 * q + i;
            put_bf16(c.s + S_H1, km_off(r, j, HID), fmaxf(v[i] + p[OFF_B1 + j], 0.f));
        }
    }
    // layer 2
    if (!run_gemm(c.tmem, 0, c.sbase + S_H1, c.sbase + S_W2, HID, HID, c.mbar, c.phase, c.abort_flag)) return false;
    for (int q = 0; q < HID / 16; q++) {
        float v[16];
        tmem_ld16(lane_addr + 16 * q, v);
#pragma unroll
        for (int i = 0; i < 16; i++) {
            int j = 16 * q + i;
            put_bf16(c.s + S_H2, km_off(r, j, HID), fmaxf(v[i] + p[OFF_B2 + j], 0.f));
        }
    }
    // layer 3 (N padded to 16)
    if (!run_gemm(c.tmem, 64, c.sbase + S_H2, c.sbase + S_W3, N3, HID, c.mbar, c.phase, c.abort_flag)) return false;
    {
        float v[16];
        tmem_ld16(lane_addr + 64, v);
        for (int o = 0; o < OUT; o++) y[o] = v[o] + p[OFF_B3 + o];
    }
    return true;
}

__device__ bool setup(Ctx& c, unsigned char* smem, uint32_t* s_tmem, unsigned long long* s_mbar, int* s_abort) {
    c.s = smem;
    c.sbase = smem_u32(smem);
    c.abort_flag = s_abort;
    const int warp = threadIdx.x >> 5;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(smem_u32(s_tmem)), "r"(TMEM_COLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(s_mbar)) : "memory");
        *s_abort = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    c.tmem = *s_tmem;
    c.mbar = smem_u32(s_mbar);
    c.phase = 0;
    return true;
}

__device__ void teardown(Ctx& c) {
    tc_fence_before();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(c.tmem), "r"(TMEM_COLS) : "memory");
}

__global__ void __launch_bounds__(TILE) k_mlp_forward(MlpArgs g) {
    extern __shared__ __align__(1024) unsigned char mlp_smem[];
    __shared__ uint32_t s_tmem;
    __shared__ __align__(8) unsigned long long s_mbar;
    __shared__ int s_abort;
    Ctx c;
    setup(c, mlp_smem, &s_tmem, &s_mbar, &s_abort);
    stage_rows(c.s + S_W1, g.wb + WB_W1, HID, K1);
    stage_rows(c.s + S_W2, g.wb + WB_W2, HID, HID);
    stage_rows(c.s + S_W3, g.wb + WB_W3, N3, HID);
    const int n = g.nptr ? min(*g.nptr, g.n) : g.n;
    for (int t = blockIdx.x; t * TILE < n; t += gridDim.x) {
        float y[OUT];
        if (!forward_tile(c, g, t * TILE, n, y, nullptr)) break;
        const int row = t * TILE + threadIdx.x;
        if (row < n)
            for (int o = 0; o < OUT; o++) g.out[(size_t)row * OUT + o] = y[o] * g.p[OFF_OSCALE + o];
    }
    if (s_abort && threadIdx.x == 0) atomicCAS(g.status, 0, JG_ERR_TIMEOUT);
    teardown(c);
}

// Forward + backward over tiles; gradients of the summed squared error / (3 n) of the
// normalised outputs, accumulated into g.grad with FP32 atomics.
__global__ void __launch_bounds__(TILE) k_mlp_train(MlpArgs g) {
    extern __shared__ __align__(1024) unsigned char mlp_smem[];
    __shared__ uint32_t s_tmem;
    __shared__ __align__(8) unsigned long long s_mbar;
    __shared__ int s_abort;
    __shared__ float s_dy[TILE][OUT];
    __shared__ float s_db1[HID], s_db2[HID];
    __shared__ float s_loss;
    Ctx c;
    setup(c, mlp_smem, &s_tmem, &s_mbar, &s_abort);
    stage_rows(c.s + S_W1, g.wb + WB_W1, HID, K1);
    stage_rows(c.s + S_W2, g.wb + WB_W2, HID, HID);
    stage_rows(c.s + S_W3, g.wb + WB_W3, N3, HID);
    stage_rows(c.s + S_W3T, g.wb + WB_W3T, HID, N3);
    stage_rows(c.s + S_W2T, g.wb + WB_W2T, HID, HID);
    const int r = threadIdx.x, warp = r >> 5, lane = r & 31;
    const int n = g.n;
    const float inv3n = 1.0f / (3.0f * (float)n);
    const uint32_t lane_addr = c.tmem + ((uint32_t)(32 * warp) << 16);
    if (r < HID) { s_db1[r] = 0.f; s_db2[r] = 0.f; }
    if (r == 0) s_loss = 0.f;
    for (int t = blockIdx.x; t * TILE < n; t += gridDim.x) {
        const int r0 = t * TILE;
        const bool valid = r0 + r < n;
        float y[OUT], xr[K1];
        if (!forward_tile(c, g, r0, n, y, xr)) break;
        // output error and dY (normalised units)
        float dy[OUT], se = 0.f;
        for (int o = 0; o < OUT; o++) {
            float e = valid ? y[o] - g.T[(size_t)(r0 + r) * OUT + o] / g.p[OFF_OSCALE + o] : 0.f;
            se += e * e;
            dy[o] = 2.0f * e * inv3n;
            s_dy[r][o] = dy[o];
        }
        for (int off = 16; off > 0; off >>= 1) se += __shfl_xor_sync(0xffffffffu, se, off);
        if (lane == 0) atomicAdd(&s_loss, se);
        for (int k = 0; k < N3; k++) put_bf16(c.s + S_DY, km_off(r, k, N3), k < OUT ? dy[k] : 0.f);
        // b3 and W3 gradients on the CUDA cores (3 x 64 outer-product sum)
        for (int o = 0; o < OUT; o++) {
            float sdy = dy[o];
            for (int off = 16; off > 0; off >>= 1) sdy += __shfl_xor_sync(0xffffffffu, sdy, off);
            if (lane == 0) atomicAdd(&g.grad[OFF_B3 + o], sdy);
        }
        __syncthreads();
        for (int q = r; q < OUT * HID; q += blockDim.x) {
            int o = q / HID, j = q - o * HID;
            float acc = 0.f;
            for (int s = 0; s < TILE; s++) acc += s_dy[s][o] * get_bf16(c.s + S_H2, km_off(s, j, HID));
            atomicAdd(&g.grad[OFF_W3 + o * HID + j], acc);
        }
        // dH2 = dY W3 -> dZ2 = dH2 * [H2 > 0]
        if (!run_gemm(c.tmem, 0, c.sbase + S_DY, c.sbase + S_W3T, HID, N3, c.mbar, c.phase, c.abort_flag)) break;
        for (int q = 0; q < HID / 16; q++) {
            float v[16];
            tmem_ld16(lane_addr + 16 * q, v);
#pragma unroll
            for (int i = 0; i < 16; i++) {
                int j = 16 * q + i;
                float dz = get_bf16(c.s + S_H2, km_off(r, j, HID)) > 0.f ? v[i] : 0.f;
                atomicAdd(&s_db2[j], dz);
                __nv_bfloat16 b = __float2bfloat16_rn(dz);
                *(__nv_bfloat16*)(c.s + S_DZ2 + km_off(r, j, HID)) = b;
                *(__nv_bfloat16*)(c.s + S_A + km_off(j, r, TILE)) = b;          // dZ2^T rows 0..63
            }
        }
        // dH1 = dZ2 W2 -> dZ1 = dH1 * [H1 > 0]
        if (!run_gemm(c.tmem, 0, c.sbase + S_DZ2, c.sbase + S_W2T, HID, HID, c.mbar, c.phase, c.abort_flag)) break;
        for (int q = 0; q < HID / 16; q++) {
            float v[16];
            tmem_ld16(lane_addr + 16 * q, v);
#pragma unroll
            for (int i = 0; i < 16; i++) {
                int j = 16 * q + i;
                float h1 = get_bf16(c.s + S_H1, km_off(r, j, HID));
                float dz = h1 > 0.f ? v[i] : 0.f;
                atomicAdd(&s_db1[j], dz);
                put_bf16(c.s + S_A, km_off(HID + j, r, TILE), dz);             // dZ1^T rows 64..127
                *(__nv_bfloat16*)(c.s + S_B + km_off(j, r, TILE)) = __float2bfloat16_rn(h1);  // H1^T rows 0..63
            }
        }
        for (int f = 0; f < K1; f++) put_bf16(c.s + S_B, km_off(HID + f, r, TILE), xr[f]);  // X^T rows 64..95
        // [dW2 | . ; . | dW1] = [dZ2^T ; dZ1^T] [H1 | X]
        if (!run_gemm(c.tmem, 0, c.sbase + S_A, c.sbase + S_B, 96, TILE, c.mbar, c.phase, c.abort_flag)) break;
        if (warp < 2) {
            const int i = r;  // dW2 row
            for (int q = 0; q < HID / 16; q++) {
                float v[16];
                tmem_ld16(lane_addr + 16 * q, v);
#pragma unroll
                for (int k = 0; k < 16; k++) atomicAdd(&g.grad[OFF_W2 + i * HID + 16 * q + k], v[k]);
            }
        } else {
            const int j = r - HID;  // dW1 row
            for (int q = 0; q < 2; q++) {
                float v[16];
                tmem_ld16(lane_addr + HID + 16 * q, v);
#pragma unroll
                for (int k = 0; k < 16; k++) {
                    int f = 16 * q + k;
                    if (f < IN) atomicAdd(&g.grad[OFF_W1 + j * IN + f], v[k]);
                }
            }
        }
    }
    __syncthreads();
    if (r < HID) {
        atomicAdd(&g.grad[OFF_B1 + r], s_db1[r]);
        atomicAdd(&g.grad[OFF_B2 + r], s_db2[r]);
    }
    if (r == 0) atomicAdd(g.loss, s_loss);
    if (s_abort && threadIdx.x == 0) atomicCAS(g.status, 0, JG_ERR_TIMEOUT);
    teardown(c);
}

// BF16 operand copies from the FP32 parameters.
__global__ void k_mlp_refresh(const float* p, __nv_bfloat16* wb) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < WB_TOTAL; i += gridDim.x * blockDim.x) {
        float v = 0.f;
        if (i < WB_W2) { int r = i / K1, k = i - r * K1; v = k < IN ? p[OFF_W1 + r * IN + k] : 0.f; }
        else if (i < WB_W3) { int q = i - WB_W2; v = p[OFF_W2 + q]; }
        else if (i < WB_W3T) { int q = i - WB_W3, r = q / HID, k = q - r * HID; v = r < OUT ? p[OFF_W3 + r * HID + k] : 0.f; }
        else if (i < WB_W2T) { int q = i - WB_W3T, j = q / N3, o = q - j * N3; v = o < OUT ? p[OFF_W3 + o * HID + j] : 0.f; }
        else { int q = i - WB_W2T, j = q / HID, k = q - j * HID; v = p[OFF_W2 + k * HID + j]; }
        wb[i] = __float2bfloat16_rn(v);
    }
}

__global__ void k_mlp_adam(float* p, const float* g, float* m, float* v, float lr, float c1, float c2) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NW; i += gridDim.x * blockDim.x) {
        float gi = g[i];
        float mi = b1 * m[i] + (1.0f - b1) * gi;
        float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi; v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

// Features of every contact created by this step's merge (NewContact flag), with the
// arbiter and slot they belong to.
__global__ void k_mlp_features(WorldDev w, float* feat, int2* fidx, int* fcount, int cap) {
    const ArbStore& A = w.arb[w.cur];
    const int narb = min(w.ctr->narb, w.cap_arb), ca = w.cap_arb;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < narb; a += gridDim.x * blockDim.x) {
        int4 info = A.info[a];
        int usage = info.x & 15;
        if (!usage) continue;
        int2 bb = A.body[a];
        for (int k = 0; k < 4; k++) {
            if (!(usage & (1 << k))) continue;
            int i = k * ca + a;
            float4 ct2 = A.ct2[i];
            if (!(__float_as_int(ct2.w) & 2)) continue;
            int e = atomicAdd(fcount, 1);
            if (e >= cap) continue;
            SBody B1 = w.body[bb.x], B2 = w.body[bb.y];
            v3 n = mk3(A.cn[i]), t1 = mk3(A.ct1[i]), t2 = mk3(ct2);
            v3 r1 = mk3(A.cr1[i]), r2 = mk3(A.cr2[i]);
            v3 dv = (mk3(B2.v) + cross(mk3(B2.w), r2)) - (mk3(B1.v) + cross(mk3(B1.w), r1));
            v3 p1 = r1 + mk3(w.pos[bb.x]), p2 = r2 + mk3(w.pos[bb.y]);
            float* f = feat + (size_t)e * IN;
            f[0] = n.x; f[1] = n.y; f[2] = n.z;
            f[3] = t1.x; f[4] = t1.y; f[5] = t1.z;
            f[6] = dot(n, dv); f[7] = dot(t1, dv); f[8] = dot(t2, dv);
            f[9] = dot(p1 - p2, n);
            f[10] = B1.v.w; f[11] = B2.v.w;
            f[12] = B1.i0.x; f[13] = B1.i0.w; f[14] = B1.i1.y;
            f[15] = B2.i0.x; f[16] = B2.i0.w; f[17] = B2.i1.y;
            f[18] = r1.x; f[19] = r1.y; f[20] = r1.z;
            f[21] = r2.x; f[22] = r2.y; f[23] = r2.z;
            fidx[e] = make_int2(a, k);
        }
    }
}

// Writes the predicted impulses into the new contacts' accumulators, projected onto the
// solver's admissible set (normal >= 0, friction inside the box of the friction cone).
__global__ void k_mlp_apply(WorldDev w, const float* pred, const int2* fidx, const int* fcount, int cap) {
    const ArbStore& A = w.arb[w.cur];
    const int n = min(*fcount, cap), ca = w.cap_arb;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        int2 ak = fidx[e];
        int i = ak.y * ca + ak.x;
        float an = fmaxf(pred[3 * e], 0.f);
        float mu = A.mat[ak.x].x;
        float lim = mu * an;
        float t1 = fminf(fmaxf(pred[3 * e + 1], -lim), lim), t2 = fminf(fmaxf(pred[3 * e + 2], -lim), lim);
        if (!isfinite(an) || !isfinite(t1) || !isfinite(t2)) continue;
        float4 c = A.cacc[i];
        A.cacc[i] = make_float4(an, t1, t2, c.w);
    }
}

// No warm start at all: every accumulated impulse starts the step at zero.
__global__ void k_zero_warmstart(WorldDev w) {
    const ArbStore& A = w.arb[w.cur];
    const int narb = min(w.ctr->narb, w.cap_arb), ca = w.cap_arb;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < narb; a += gridDim.x * blockDim.x)
        for (int k = 0; k < 4; k++) {
            float4 c = A.cacc[k * ca + a];
            A.cacc[k * ca + a] = make_float4(0.f, 0.f, 0.f, c.w);
        }
}

struct Mlp {
    float *p = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr, *loss = nullptr;
    __nv_bfloat16* wb = nullptr;
    int* status = nullptr;
    // per-step contact features
    float *feat = nullptr, *pred = nullptr, *tgt = nullptr;
    int2* fidx = nullptr;
    int* fcount = nullptr;
    int cap = 0;
    // host I/O staging
    float *x = nullptr, *t = nullptr, *out = nullptr;
    int io_cap = 0;
    bool loaded = false, collect = false, recorded = false;
    int adam_t = 0;
};

int mlp_fail(cudaError_t e, const char* what) {
    std::string s = std::string(what) + ": " + cudaGetErrorString(e);
    jg_set_error(s.c_str());
    return JG_ERR_CUDA;
}
#define MCK(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) return mlp_fail(_e, #x); } while (0)

size_t fwd_smem() { return (size_t)S_FWD_END; }
size_t train_smem() { return (size_t)S_TRAIN_END; }

int mlp_get(jg_world* w, Mlp** out) {
    void*& slot = jg_world_mlp(w);
    if (!slot) {
        Mlp* m = new Mlp();
        WorldDev& d = jg_world_dev(w);
        MCK(cudaMalloc((void**)&m->p, sizeof(float) * NPARAM));
        MCK(cudaMalloc((void**)&m->m, sizeof(float) * NW));
        MCK(cudaMalloc((void**)&m->v, sizeof(float) * NW));
        MCK(cudaMalloc((void**)&m->grad, sizeof(float) * NW));
        MCK(cudaMalloc((void**)&m->loss, sizeof(float) * 2));
        MCK(cudaMalloc((void**)&m->status, sizeof(int)));
        MCK(cudaMalloc((void**)&m->wb, sizeof(__nv_bfloat16) * WB_TOTAL));
        m->cap = d.cap_arb;
        MCK(cudaMalloc((void**)&m->feat, sizeof(float) * IN * (size_t)m->cap));
        MCK(cudaMalloc((void**)&m->pred, sizeof(float) * OUT * (size_t)m->cap));
        MCK(cudaMalloc((void**)&m->tgt, sizeof(float) * OUT * (size_t)m->cap));
        MCK(cudaMalloc((void**)&m->fidx, sizeof(int2) * (size_t)m->cap));
        MCK(cudaMalloc((void**)&m->fcount, sizeof(int)));
        cudaStream_t s = jg_world_stream(w);
        MCK(cudaMemsetAsync(m->p, 0, sizeof(float) * NPARAM, s));
        MCK(cudaMemsetAsync(m->m, 0, sizeof(float) * NW, s));
        MCK(cudaMemsetAsync(m->v, 0, sizeof(float) * NW, s));
        MCK(cudaMemsetAsync(m->status, 0, sizeof(int), s));
        MCK(cudaMemsetAsync(m->fcount, 0, sizeof(int), s));
        MCK(cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fwd_smem()));
        MCK(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem()));
        slot = m;
    }
    *out = (Mlp*)slot;
    return JG_OK;
}

int ensure_io(Mlp* m, int n) {
    if (n <= m->io_cap) return JG_OK;
    cudaFree(m->x); cudaFree(m->t); cudaFree(m->out);
    m->x = m->t = m->out = nullptr;
    int c = std::max(n, 1024);
    MCK(cudaMalloc((void**)&m->x, sizeof(float) * IN * (size_t)c));
    MCK(cudaMalloc((void**)&m->t, sizeof(float) * OUT * (size_t)c));
    MCK(cudaMalloc((void**)&m->out, sizeof(float) * OUT * (size_t)c));
    m->io_cap = c;
    return JG_OK;
}

MlpArgs args(const Mlp* m) {
    MlpArgs g{};
    g.wb = m->wb; g.p = m->p; g.grad = m->grad; g.loss = m->loss; g.status = m->status;
    return g;
}

int check_status(Mlp* m, cudaStream_t s) {
    int st = 0;
    MCK(cudaMemcpyAsync(&st, m->status, sizeof(int), cudaMemcpyDeviceToHost, s));
    MCK(cudaStreamSynchronize(s));
    MCK(cudaGetLastError());
    if (st) { jg_set_error("MLP kernel reported a device error (tensor-core wait timed out)"); return st; }
    return JG_OK;
}

// Gradients (and loss) of a host minibatch into m->grad / m->loss; leaves them on device.
int run_gradients(jg_world* w, Mlp* m, const float* X, const float* T, int n) {
    cudaStream_t s = jg_world_stream(w);
    int r = ensure_io(m, n);
    if (r) return r;
    MCK(cudaMemcpyAsync(m->x, X, sizeof(float) * IN * (size_t)n, cudaMemcpyHostToDevice, s));
    MCK(cudaMemcpyAsync(m->t, T, sizeof(float) * OUT * (size_t)n, cudaMemcpyHostToDevice, s));
    MCK(cudaMemsetAsync(m->grad, 0, sizeof(float) * NW, s));
    MCK(cudaMemsetAsync(m->loss, 0, sizeof(float) * 2, s));
    MlpArgs g = args(m);
    g.X = m->x; g.T = m->t; g.n = n;
    int tiles = (n + TILE - 1) / TILE;
    k_mlp_train<<<std::min(tiles, jg_world_nsm(w)), TILE, train_smem(), s>>>(g);
    MCK(cudaGetLastError());
    return JG_OK;
}

}  // namespace

void jg_mlp_free(void* p) {
    Mlp* m = (Mlp*)p;
    if (!m) return;
    cudaFree(m->p); cudaFree(m->m); cudaFree(m->v); cudaFree(m->grad); cudaFree(m->loss); cudaFree(m->status);
    cudaFree(m->wb); cudaFree(m->feat); cudaFree(m->pred); cudaFree(m->tgt); cudaFree(m->fidx); cudaFree(m->fcount);
    cudaFree(m->x); cudaFree(m->t); cudaFree(m->out);
    delete m;
}

// Per-step hook after the arbiter merge: zero warm start, or the features of new contacts
// (for training-data collection and/or the learned warm start).  Returns the kernels
// launched.
int jg_mlp_step_hook(jg_world* w, const StepParams& sp) {
    WorldDev& d = jg_world_dev(w);
    cudaStream_t s = jg_world_stream(w);
    const int nsm = jg_world_nsm(w);
    if (sp.warm_start == JG_WARMSTART_ZERO) {
        k_zero_warmstart<<<nsm * 4, 256, 0, s>>>(d);
        return 1;
    }
    Mlp* m = (Mlp*)jg_world_mlp(w);
    if (!m) return 0;
    const bool learned = sp.warm_start == JG_WARMSTART_MLP && m->loaded;
    if (!learned && !m->collect) return 0;
    cudaMemsetAsync(m->fcount, 0, sizeof(int), s);
    k_mlp_features<<<nsm * 4, 256, 0, s>>>(d, m->feat, m->fidx, m->fcount, m->cap);
    m->recorded = true;
    if (!learned) return 1;
    MlpArgs g = args(m);
    g.X = m->feat; g.nptr = m->fcount; g.n = m->cap; g.out = m->pred;
    k_mlp_forward<<<nsm, TILE, fwd_smem(), s>>>(g);
    k_mlp_apply<<<nsm * 4, 256, 0, s>>>(d, m->pred, m->fidx, m->fcount, m->cap);
    return 3;
}

extern "C" {

int jg_mlp_load(jg_world* w, const float* params, int32_t count) {
    if (!w || !params || count != NPARAM) { jg_set_error("jg_mlp_load: expects 6006 floats"); return JG_ERR_INVALID_ARG; }
    for (int i = 0; i < count; i++) if (!std::isfinite(params[i])) return JG_ERR_NONFINITE;
    Mlp* m;
    int r = mlp_get(w, &m);
    if (r) return r;
    cudaStream_t s = jg_world_stream(w);
    MCK(cudaMemcpyAsync(m->p, params, sizeof(float) * NPARAM, cudaMemcpyHostToDevice, s));
    MCK(cudaMemsetAsync(m->m, 0, sizeof(float) * NW, s));
    MCK(cudaMemsetAsync(m->v, 0, sizeof(float) * NW, s));
    k_mlp_refresh<<<16, 256, 0, s>>>(m->p, m->wb);
    MCK(cudaStreamSynchronize(s));
    m->adam_t = 0;
    m->loaded = true;
    jg_world_set_mlp_ready(w, true);
    jg_world_invalidate_graphs(w);  // the step's launch sequence changes
    return JG_OK;
}

int jg_mlp_export(jg_world* w, float* params, int32_t capacity, int32_t* out_count) {
    if (!w || !out_count) return JG_ERR_INVALID_ARG;
    *out_count = NPARAM;
    Mlp* m = (Mlp*)jg_world_mlp(w);
    if (!m || !m->loaded) { jg_set_error("jg_mlp_export: no model loaded"); return JG_ERR_INVALID_ARG; }
    if (!params || capacity < NPARAM) return JG_OK;
    cudaStream_t s = jg_world_stream(w);
    MCK(cudaMemcpyAsync(params, m->p, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, s));
    MCK(cudaStreamSynchronize(s));
    return JG_OK;
}

int jg_mlp_predict(jg_world* w, const float* features, int32_t n, float* out) {
    if (!w || n < 0 || (n > 0 && (!features || !out))) return JG_ERR_INVALID_ARG;
    Mlp* m = (Mlp*)jg_world_mlp(w);
    if (!m || !m->loaded) { jg_set_error("jg_mlp_predict: no model loaded"); return JG_ERR_INVALID_ARG; }
    if (n == 0) return JG_OK;
    int r = ensure_io(m, n);
    if (r) return r;
    cudaStream_t s = jg_world_stream(w);
    MCK(cudaMemcpyAsync(m->x, features, sizeof(float) * IN * (size_t)n, cudaMemcpyHostToDevice, s));
    MlpArgs g = args(m);
    g.X = m->x; g.n = n; g.out = m->out;
    int tiles = (n + TILE - 1) / TILE;
    k_mlp_forward<<<std::min(tiles, jg_world_nsm(w)), TILE, fwd_smem(), s>>>(g);
    MCK(cudaGetLastError());
    MCK(cudaMemcpyAsync(out, m->out, sizeof(float) * OUT * (size_t)n, cudaMemcpyDeviceToHost, s));
    return check_status(m, s);
}

int jg_mlp_gradients(jg_world* w, const float* features, const float* targets, int32_t n, float* out_grads,
                     int32_t capacity, float* out_loss) {
    if (!w || n <= 0 || !features || !targets) return JG_ERR_INVALID_ARG;
    Mlp* m = (Mlp*)jg_world_mlp(w);
    if (!m || !m->loaded) { jg_set_error("jg_mlp_gradients: no model loaded"); return JG_ERR_INVALID_ARG; }
    int r = run_gradients(w, m, features, targets, n);
    if (r) return r;
    cudaStream_t s = jg_world_stream(w);
    if (out_grads && capacity >= NW) MCK(cudaMemcpyAsync(out_grads, m->grad, sizeof(float) * NW, cudaMemcpyDeviceToHost, s));
    float l = 0.f;
    MCK(cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, s));
    r = check_status(m, s);
    if (out_loss) *out_loss = l / (3.0f * (float)n);
    return r;
}

int jg_mlp_train_step(jg_world* w, const float* features, const float* targets, int32_t n, float lr, float* out_loss) {
    if (!w || n <= 0 || !features || !targets || !(lr > 0.f)) return JG_ERR_INVALID_ARG;
    Mlp* m = (Mlp*)jg_world_mlp(w);
    if (!m || !m->loaded) { jg_set_error("jg_mlp_train_step: no model loaded"); return JG_ERR_INVALID_ARG; }
    int r = run_gradients(w, m, features, targets, n);
    if (r) return r;
    cudaStream_t s = jg_world_stream(w);
    m->adam_t++;
    float c1 = 1.0f - std::pow(0.9f, (float)m->adam_t), c2 = 1.0f - std::pow(0.999f, (float)m->adam_t);
    k_mlp_adam<<<8, 256, 0, s>>>(m->p, m->grad, m->m, m->v, lr, c1, c2);
    k_mlp_refresh<<<16, 256, 0, s>>>(m->p, m->wb);
    float l = 0.f;
    MCK(cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, s));
    r = check_status(m, s);
    if (out_loss) *out_loss = l / (3.0f * (float)n);
    return r;
}

int jg_collect_training(jg_world* w, float* features, float* targets, int32_t capacity, int32_t* out_count) {
    if (!w || !out_count || capacity < 0) return JG_ERR_INVALID_ARG;
    Mlp* m;
    int r = mlp_get(w, &m);
    if (r) return r;
    *out_count = 0;
    const bool was = m->recorded;
    if (!m->collect) {
        // from now on every step records its new contacts and, in the solver, their
        // impulses after the first substep
        WorldDev& d = jg_world_dev(w);
        d.rec_on = 1;
        d.rec_cap = m->cap;
        d.rec_fidx = m->fidx;
        d.rec_count = m->fcount;
        d.rec_dst = jg_world_dst_index(w);
        d.rec_tgt = m->tgt;
        jg_world_invalidate_graphs(w);
        m->collect = true;
    }
    if (!was) return JG_OK;
    cudaStream_t s = jg_world_stream(w);
    int cnt = 0;
    MCK(cudaMemcpyAsync(&cnt, m->fcount, sizeof(int), cudaMemcpyDeviceToHost, s));
    MCK(cudaStreamSynchronize(s));
    cnt = std::min(cnt, m->cap);
    int k = std::min(cnt, capacity);
    if (k > 0 && features && targets) {
        MCK(cudaMemcpyAsync(features, m->feat, sizeof(float) * IN * (size_t)k, cudaMemcpyDeviceToHost, s));
        MCK(cudaMemcpyAsync(targets, m->tgt, sizeof(float) * OUT * (size_t)k, cudaMemcpyDeviceToHost, s));
    }
    MCK(cudaStreamSynchronize(s));
    MCK(cudaGetLastError());
    *out_count = features && targets ? k : cnt;
    return JG_OK;
}

}  // extern "C"
