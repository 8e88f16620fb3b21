/* ncc_tc.cu -- the correlation map on the 5th-generation tensor cores: tcgen05.mma (kind::f16, BF16 or FP16 products,
 * F32 accumulation in tensor memory), operands brought into shared memory by asynchronous bulk copies and read through
 * matrix descriptors, the accumulator read back with tcgen05.ld, scored with exact int64 window sums and reduced to the
 * per-cell map in the epilogue.
 *
 * The correlation as a GEMM. A CTA owns a tile of corners: 1024 consecutive x (X0 + 8 m + s, m < 128, s < 8) by Q
 * consecutive y (Y0 + q, q < Q; Q = 16, or 8 for templates wider than 120). Then
 *     st(X0 + 8 m + s, Y0 + q) = sum over image rows r, columns c of  A_r[m][c] * B_r[(q, s)][c]
 * with A_r[m][c] = J[r][X0 + 8 m + c] and B_r[(q, s)][c] = t[r - Y0 - q][c - s] (zero outside the template): D =
 * sum_r A_r B_r^T with M = 128, N = 8 Q, and K = the tile's Q + T_h - 1 image rows times K_row = T_w + 8 rounded up
 * to 16.
 *   A needs no im2col. Consecutive rows of A_r start 8 elements (16 bytes) apart in the image row, so a K-major,
 *   no-swizzle descriptor with 16-byte core-matrix rows, a 16-byte leading (K) offset and a 128-byte stride (M) offset
 *   reads A_r straight from the row: address(m, k) = row + 2 (8 m + k). The picture is converted to 16 bits once per
 *   search (ncc_prep), shifted so that every tile's row segment starts on a 16-byte boundary.
 *   B_r depends only on r - Y0: the band (Q + T_h - 1 blocks of 8 Q x K_row) is built once per template in the canonical
 *   core-matrix layout.
 * Pipeline: three threads drive it. Six shared-memory stages, each an image-row segment and a band block, arrive by
 * cp.async.bulk on a "full" mbarrier (expected bytes). A producer thread (warp 0) fills a stage again as soon as the
 * MMAs of its last use commit to its "empty" mbarrier. Two issuer threads (warps 1 and 2) take alternate stages, each
 * into its own accumulator: issuing a stage's MMAs takes a lone thread longer than the tensor core takes to run them,
 * so one issuer would leave it idle. Every wait is bounded by the global timer; past it the kernel records an error
 * word.
 * Epilogue: four warps cover the accumulator's 128 lanes, one row (8 x-corners by Q y-corners) a thread; at Q = 16
 * eight, two to a lane quarter, each reading half the row's columns. A thread sums the issuers' accumulators for its
 * row. Per corner: st = acc - J(x, y) sum t' (the reference's st is relative to the corner's first pixel), times the
 * corner's factor 1 / sqrt(norm var) from ncc_prep (0 for a near-blank window: the exact integer rule), the best
 * per 16 x 16 cell by value then scan order, merged across tiles by a 64-bit atomicMax on (ordered score, inverted scan
 * index). */
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "vtg_ncc.cuh"

#define TC_M 128
#define TC_QMAX 16 /* y-corners of a tile, at most */
#define TC_XS (8 * TC_M) /* x-corners of a tile */
#define TC_STAGES 6
#ifndef TC_ISSUERS
#define TC_ISSUERS 2 /* MMA-issuing threads, each with its own accumulator, taking every TC_ISSUERS-th stage */
#endif
#define TC_WAIT_NS 2000000000ull /* a wait gives up after 2 s of the global timer */
#define TC_MAX_KROW 144          /* T_w <= 128 */

static inline int tc_krow(int tw) { return ((tw + 8 + 15) / 16) * 16; }

/* y-corners of a tile (N = 8 Q). An MMA reads its A (4 KB) and B (16 N bytes) from shared memory at 128 bytes a cycle
 * and multiplies for N / 2 cycles, so below N = 128 the shared-memory reads bound it. Q = 16 while six stages of it fit
 * the shared memory (K_row <= 128), else 8. The band's zero rows (Q - 1 of every Q + th - 1 image rows) cost less than
 * the reads they save. */
#ifndef TC_Q_BIG
#define TC_Q_BIG 16
#endif
static inline int tc_q(int tw, int th)
{
    (void)th;
    return TC_Q_BIG == 16 && tc_krow(tw) > 128 ? 8 : TC_Q_BIG;
}

/* the band at its largest tile height: enough for either */
size_t vtg_ncc_band_bytes(int tw, int th) { return (size_t)(TC_QMAX + th - 1) * 8 * TC_QMAX * tc_krow(tw) * sizeof(uint16_t); }

/* The 16-bit picture: rows up to h + TC_QMAX + T_h (zeros past the picture), TC_XS-aligned tiles plus the last K row. */
static inline int conv_pitch(int w) { return ((w + TC_XS - 1) / TC_XS) * TC_XS + TC_MAX_KROW; }

size_t vtg_ncc_conv_elems(int max_w, int max_h, int max_th) { return (size_t)conv_pitch(max_w) * (size_t)(max_h + TC_QMAX + max_th); }

/* The corners' factors: rows of whole tiles (TC_XS corners), so a tile's factor loads stay inside its row. */
size_t vtg_ncc_fac_elems(int max_w, int max_h) { return (size_t)((max_w + TC_XS - 1) / TC_XS) * TC_XS * (size_t)max_h; }

/* ---- the band ---- */

__device__ __forceinline__ uint16_t to16(float v, int kind)
{
    return kind == VTG_NCC_BF16 ? __bfloat16_as_ushort(__float2bfloat16_rn(v)) : __half_as_ushort(__float2half_rn(v));
}

__device__ __forceinline__ float from16(uint16_t v, int kind)
{
    return kind == VTG_NCC_BF16 ? __bfloat162float(__ushort_as_bfloat16(v)) : __half2float(__ushort_as_half(v));
}

/* Band block k (image row Y0 + k of a tile), element (n = 8 q + s, c) at core matrix (c / 8, n / 8), row n % 8, column
 * c % 8: core matrices of 8 x 8 elements (128 bytes), K-chunks of 8 columns N / 8 matrices apart. */
__global__ void ncc_band_kernel(const float *__restrict__ app, int tw, int th, int kind, int krow, int rows, int nq,
                                uint16_t *__restrict__ band)
{
    const int N = 8 * nq;
    const size_t per = (size_t)N * krow;
    const size_t total = per * rows;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(idx / per);
        const int rem = (int)(idx - (size_t)k * per);
        const int n = rem / krow, c = rem - n * krow;
        const int q = n >> 3, s = n & 7;
        const int i = k - q, j = c - s;
        const float v = (i >= 0 && i < th && j >= 0 && j < tw) ? app[i * tw + j] : 0.0f;
        const size_t off = (size_t)k * per + ((size_t)(c >> 3) * (N / 8) + (n >> 3)) * 64 + (n & 7) * 8 + (c & 7);
        band[off] = to16(v, kind);
    }
}

/* The sum of the template as the tensor cores see it (its rounded values), in double. */
__global__ void ncc_band_sum(const float *__restrict__ app, int count, int kind, float *__restrict__ out)
{
    __shared__ double s[256];
    double a = 0.0;
    for (int i = threadIdx.x; i < count; i += blockDim.x)
        a += (double)from16(to16(app[i], kind), kind);
    s[threadIdx.x] = a;
    __syncthreads();
    for (int h = 128; h >= 1; h >>= 1) {
        if (threadIdx.x < h)
            s[threadIdx.x] += s[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        *out = (float)s[0];
}

cudaError_t vtg_launch_ncc_band(const float *app, int tw, int th, int kind, uint16_t *band, float *sum_t, cudaStream_t st)
{
    const int q = tc_q(tw, th), krow = tc_krow(tw), rows = q + th - 1;
    const size_t total = (size_t)8 * q * krow * rows;
    const int blocks = (int)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
    ncc_band_kernel<<<blocks, 256, 0, st>>>(app, tw, th, kind, krow, rows, q, band);
    ncc_band_sum<<<1, 256, 0, st>>>(app, tw * th, kind, sum_t);
    return cudaGetLastError();
}

/* ---- per-search preparation ---- */

/* conv[r][i] = 16-bit J[r][x0 + i] (zero past the picture), for rows 0 .. rows - 1 and columns 0 .. cpitch - 1: the
 * CTA (bx, by) of 256 threads converts row by, eight elements a thread and one 16-byte store (cpitch is a multiple of 8
 * and rows start 16-byte aligned: 2 cpitch = 2048 tiles_x + 288 bytes). */
template <int KIND>
__device__ __forceinline__ void conv_cta(const uint8_t *__restrict__ plane, int pitch, int w, int h, int x0, int rows,
                                         int cpitch, uint16_t *__restrict__ conv, int bx, int by)
{
    const int r = by, i0 = 8 * (bx * 256 + (int)threadIdx.x);
    if (r >= rows || i0 >= cpitch)
        return;
    uint32_t o[4];
#pragma unroll
    for (int e = 0; e < 4; e++) {
        uint32_t pr = 0;
#pragma unroll
        for (int f = 0; f < 2; f++) {
            const int x = x0 + i0 + 2 * e + f;
            const float v = (r < h && x < w) ? (float)__ldg(plane + (size_t)r * pitch + x) : 0.0f;
            pr |= (uint32_t)to16(v, KIND) << (16 * f);
        }
        o[e] = pr;
    }
    *reinterpret_cast<uint4 *>(conv + (size_t)r * cpitch + i0) = make_uint4(o[0], o[1], o[2], o[3]);
}

/* fac[(y - y0) fpitch + (x - x0)] = 1 / sqrt(norm var) from the corner's exact window sums; 0 for a near-blank window
 * (n var <= n norm / 16) or norm <= 0 -- the reference's rule (src/kern/track.c:203-205) on exact integers.
 * The sums come straight from the bytes, a tile of btx x BP_TY corners a CTA (btx = bp_tx(T_w)), one thread a column
 * of the tile:
 *   - down its column, running sums over the template's T_h rows for the tile's BP_TY corner rows (registers);
 *   - across the columns, each row's prefix sums: a shuffle scan in the warp, the earlier warps' totals added from
 *     shared memory;
 *   - a corner's window sums are then P(x + T_w) - P(x), consecutive lanes on consecutive corners.
 * Bytes keep every window sum in 32 bits (sum J^2 <= 255^2 x 128^2 < 2^31). A row's prefix of J^2 may pass 2^32, so
 * the prefixes are unsigned and wrap: their differences are still exact. n var is formed in 64 bits. */
#ifndef BP_TY
#define BP_TY 16 /* corner rows a CTA: a multiple of the 8 warps, each warp writing rows warp, warp + 8, .. */
#endif
/* corners a CTA across: the most, a multiple of 32, whose columns (+ T_w - 1) fit the CTA's 256 threads */
static inline int bp_tx(int tw) { return ((257 - tw) / 32) * 32; }
__device__ void box_cta(const uint8_t *__restrict__ plane, int pitch, const NccPrm &p, int fw, int fpitch, int btx,
                        float *__restrict__ fac, int bx, int by)
{
    __shared__ unsigned P1[BP_TY][257], P2[BP_TY][257]; /* P[r][c]: columns 0 .. c - 1 of row r */
    __shared__ unsigned t1[8][BP_TY], t2[8][BP_TY];     /* each warp's column totals, then the earlier warps' */
    const int fh = p.y1 - p.y0 + 1;
    const int tx0 = bx * btx, ty0 = by * BP_TY;
    const int nx = min(btx, fw - tx0), ny = min(BP_TY, fh - ty0);
    const int c = threadIdx.x, lane = c & 31, warp = c >> 5;
    const int ncol = nx + p.tw - 1; /* <= 256 */
    unsigned a[BP_TY], b[BP_TY];
    if (c < ncol) {
        const uint8_t *col = plane + (size_t)(p.y0 + ty0) * pitch + (p.x0 + tx0 + c);
        unsigned sa = 0, sb = 0;
#pragma unroll 8
        for (int i = 0; i < p.th; i++) {
            const unsigned v = __ldg(col + (size_t)i * pitch);
            sa += v;
            sb += v * v;
        }
        a[0] = sa;
        b[0] = sb;
#pragma unroll
        for (int r = 1; r < BP_TY; r++) {
            if (r < ny) {
                const unsigned o = __ldg(col + (size_t)(r - 1) * pitch), n = __ldg(col + (size_t)(r - 1 + p.th) * pitch);
                sa += n - o;
                sb += n * n - o * o;
            }
            a[r] = sa;
            b[r] = sb;
        }
    } else {
#pragma unroll
        for (int r = 0; r < BP_TY; r++)
            a[r] = b[r] = 0u;
    }
    /* inclusive scans across the warp's 32 columns */
#pragma unroll
    for (int sh = 1; sh < 32; sh <<= 1)
#pragma unroll
        for (int r = 0; r < BP_TY; r++) {
            const unsigned ua = __shfl_up_sync(VTG_FULL, a[r], sh), ub = __shfl_up_sync(VTG_FULL, b[r], sh);
            if (lane >= sh) {
                a[r] += ua;
                b[r] += ub;
            }
        }
    if (lane == 31)
#pragma unroll
        for (int r = 0; r < BP_TY; r++) {
            t1[warp][r] = a[r];
            t2[warp][r] = b[r];
        }
    __syncthreads();
    if (c < 2 * BP_TY) { /* each (row, table): the totals of the warps before, in place */
        unsigned(*t)[BP_TY] = c < BP_TY ? t1 : t2;
        const int r = c % BP_TY;
        unsigned run = 0;
        for (int w = 0; w < 8; w++) {
            const unsigned v = t[w][r];
            t[w][r] = run;
            run += v;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < BP_TY; r++) {
        P1[r][c + 1] = t1[warp][r] + a[r];
        P2[r][c + 1] = t2[warp][r] + b[r];
        if (c == 0) {
            P1[r][0] = 0u;
            P2[r][0] = 0u;
        }
    }
    __syncthreads();
    /* warp w writes corner rows w, w + 8, ..; its lanes consecutive corners (btx is a multiple of 32) */
    for (int r = warp; r < ny; r += 8) {
        float *frow = fac + (size_t)(ty0 + r) * fpitch + tx0;
#pragma unroll 1
        for (int x = lane; x < nx; x += 32) {
            const long long s1 = (long long)(P1[r][x + p.tw] - P1[r][x]), s2 = (long long)(P2[r][x + p.tw] - P2[r][x]);
            const long long nvar = (long long)p.n * s2 - s1 * s1;
            /* 1 / sqrt(norm var) = sqrt(n / norm) / sqrt(n var) */
            frow[x] = (nvar <= p.nthr || p.norm <= 0.0f) ? 0.0f : p.rnorm * rsqrtf((float)nvar);
        }
    }
}

/* The map's preparation in one launch of 256-thread CTAs: the first nbox sum the windows (the longer work, so they
 * start first), the rest convert the picture, and those also zero the cells' words the map merges into. The two jobs
 * are independent and run side by side. */
template <int KIND>
__global__ void __launch_bounds__(256) ncc_prep(const uint8_t *__restrict__ plane, int pitch, NccPrm p, int fw, int fpitch,
                                                int btx, int bgx, int nbox, float *__restrict__ fac, int rows, int cpitch,
                                                int cgx, uint16_t *__restrict__ conv, unsigned long long *__restrict__ cellw,
                                                int cells)
{
    vtg_grid_launch_dependents(); /* the map may start its setup as this launch's last CTAs run */
    const int b = (int)blockIdx.x;
    if (b < nbox) {
        box_cta(plane, pitch, p, fw, fpitch, btx, fac, b % bgx, b / bgx);
        return;
    }
    const int k = b - nbox, g = k * 256 + (int)threadIdx.x;
    if (g < cells)
        cellw[g] = 0ull;
    conv_cta<KIND>(plane, pitch, p.w, p.h, p.x0, rows, cpitch, conv, k % cgx, k / cgx);
}

/* ---- PTX helpers ---- */

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

/* A tcgen05 shared-memory matrix descriptor, no swizzle: start, leading (K) and stride (M/N) byte offsets, all in
 * 16-byte units, and the fixed version bits 46-48 = 0b001. */
__device__ __forceinline__ uint64_t mdesc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}

__device__ __forceinline__ uint64_t globaltimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

/* Bounded wait on an mbarrier phase: true when the phase with this parity completed, false after TC_WAIT_NS. */
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity)
{
    const uint64_t t0 = globaltimer();
    for (;;) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done)
                     : "r"(a), "r"(parity), "r"(100000u)
                     : "memory");
        if (done)
            return true;
        if (globaltimer() - t0 > TC_WAIT_NS)
            return false;
    }
}

/* Arms a stage's full barrier for `bytes` and brings its two operands in by bulk copy. */
__device__ __forceinline__ void tc_fill(uint32_t mbar, uint32_t dst_a, const void *src_a, uint32_t bytes_a, uint32_t dst_b,
                                        const void *src_b, uint32_t bytes_b)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes_a + bytes_b) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst_a),
                 "l"(src_a), "r"(bytes_a), "r"(mbar)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst_b),
                 "l"(src_b), "r"(bytes_b), "r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(
                     tmem_d),
                 "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
                 : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

/* 16 consecutive accumulator columns of the thread's row (lane = row within the warp's 32), not yet waited for */
__device__ __forceinline__ void tc_ld16(uint32_t taddr, uint32_t (&r)[16])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
                 "%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
}

/* A cell's candidate as one orderable word: higher score first, then the earlier corner in scan order. 0: none. */
__device__ __forceinline__ unsigned long long cell_word(float v, int key)
{
    unsigned u = __float_as_uint(v);
    u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    return ((unsigned long long)u << 32) | (unsigned long long)(0xFFFFFFFFu - (unsigned)key);
}

/* ---- the map ---- */

/* Tensor-memory columns a CTA allocates: the issuers' accumulators (8 Q columns each), rounded up to a power of two
 * of at least 32 as tcgen05.alloc requires. */
__host__ __device__ constexpr uint32_t tc_cols(int q)
{
    return 8u * q * TC_ISSUERS <= 32u ? 32u : 8u * q * TC_ISSUERS <= 64u ? 64u : 8u * q * TC_ISSUERS <= 128u ? 128u
           : 8u * q * TC_ISSUERS <= 256u ? 256u : 512u;
}
static_assert(8 * TC_QMAX * TC_ISSUERS <= 512, "the accumulators fit the tensor memory");
static_assert(TC_ISSUERS >= 1 && TC_ISSUERS <= 3, "issuers are warps 1 .. 3 of the CTA's four");

struct TcSmem {
    uint32_t a_bytes, b_bytes, stage_bytes, total;
};

static TcSmem tc_smem(int krow, int q)
{
    TcSmem s;
    s.a_bytes = (uint32_t)(((TC_XS + krow) * 2 + 127) & ~127);
    s.b_bytes = (uint32_t)(8 * q * krow * 2);
    s.stage_bytes = s.a_bytes + s.b_bytes;
    s.total = TC_STAGES * s.stage_bytes + 256; /* + mbarriers and the tensor-memory address */
    return s;
}

/* Threads of a CTA: four warps cover the accumulator's 128 lanes; at Q = 16 eight, two to a lane quarter, each warp
 * of a pair reading half the columns. chunks: 16-column blocks a thread reads. */
template <int Q> struct TcShape {
    static constexpr int threads = Q == 16 ? 256 : 128;
    static constexpr int halves = threads / 128;
    static constexpr int chunks = Q / 2 / halves;
};

template <int KIND, int Q>
__global__ void __launch_bounds__(TcShape<Q>::threads, 1) ncc_map_tc(NccPrm p, const uint16_t *__restrict__ band, int krow, int tiles_x,
                                                     uint32_t a_bytes, uint32_t stage_bytes,
                                                     const uint16_t *__restrict__ conv, int cpitch,
                                                     const float *__restrict__ fac, int fpitch,
                                                     unsigned long long *__restrict__ cellw, int *__restrict__ err)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    vtg_grid_launch_dependents(); /* the top-8 pass may take the SMs this launch leaves free and wait there */
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
    const int Y0 = p.y0 + ty * Q;
    const int nk = Q + p.th - 1;
    const int kchunks = krow / 16;
    uint8_t *ctl = smem + TC_STAGES * stage_bytes;
    const uint32_t full0 = smem_u32(ctl), empty0 = full0 + 8 * TC_STAGES;
    uint32_t *tmem_slot = (uint32_t *)(ctl + 16 * TC_STAGES);
    /* [0]: stages filled; [1 + i]: 1 + the last stage issuer i committed (0: none) */
    int *issued = (int *)(ctl + 16 * TC_STAGES + 8);
    const uint32_t a_copy = (uint32_t)((TC_XS + krow) * 2), b_copy = (uint32_t)((8 * Q) * krow * 2);

    if (tid == 0) {
        for (int s = 0; s < TC_STAGES; s++) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(tc_cols(Q))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    /* Launched as a programmatic dependent of the preparation, the CTA got here (barriers, tensor memory) while that
     * drained; everything below reads what it wrote (the 16-bit rows, the factors, the cells' reset), with ordinary
     * coherent loads: that data was not read-only while this kernel ran. */
    vtg_grid_dependency_wait();

    /* The epilogue's inputs, loaded before the MMAs start: they arrive while those run. Thread
     * (quad, lane) owns accumulator row m = 32 quad + lane, corners X0 + 8 m + s, and of its y-corners the pair half of
     * the CTA's reads: 2 chunks each. A y-corner's eight picture values (the converted row holds the bytes exactly) and
     * eight factors are one 16-byte and two 16-byte loads. */
    constexpr int CH = TcShape<Q>::chunks;
    const int m = (warp & 3) * 32 + lane, c0 = (warp >> 2) * CH;
    const int xr = tx * TC_XS + 8 * m; /* x - x0 of the thread's first corner */
    const int fh = p.y1 - p.y0 + 1;
    uint4 jr[2 * CH];
    float4 fr[4 * CH];
#pragma unroll
    for (int i = 0; i < 2 * CH; i++) {
        const int yr = ty * Q + 2 * c0 + i;
        if (yr < fh) {
            jr[i] = __ldca(reinterpret_cast<const uint4 *>(conv + (size_t)(p.y0 + yr) * cpitch + xr));
            fr[2 * i] = __ldca(reinterpret_cast<const float4 *>(fac + (size_t)yr * fpitch + xr));
            fr[2 * i + 1] = __ldca(reinterpret_cast<const float4 *>(fac + (size_t)yr * fpitch + xr + 4));
        } else {
            jr[i] = make_uint4(0u, 0u, 0u, 0u);
            fr[2 * i] = fr[2 * i + 1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    }

    const int fmt = KIND == VTG_NCC_BF16 ? 1 : 0;
    const uint32_t idesc = (1u << 4) | ((uint32_t)fmt << 7) | ((uint32_t)fmt << 10) | ((uint32_t)((8 * Q) >> 3) << 17) |
                           ((uint32_t)(TC_M >> 4) << 24);
    int good = 1;
    /* conv row r holds picture row r from column p.x0 on: this tile's segment starts at column tx * TC_XS */
    const uint16_t *arow = conv + (size_t)Y0 * cpitch + (size_t)tx * TC_XS;
    if (warp == 0 && lane == 0) {
        /* the producer: stage k % TC_STAGES is filled with image row Y0 + k and band block k once the MMAs of its
         * previous use have completed (the commit to its empty barrier) */
        int k = 0;
        for (; k < nk; k++) {
            const int s = k % TC_STAGES;
            if (k >= TC_STAGES && !mbar_wait(empty0 + 8 * s, (uint32_t)((k / TC_STAGES - 1) & 1))) {
                good = 0;
                break;
            }
            uint8_t *sa = smem + s * stage_bytes;
            tc_fill(full0 + 8 * s, smem_u32(sa), arow + (size_t)k * cpitch, a_copy, smem_u32(sa + a_bytes),
                    band + (size_t)k * (8 * Q) * krow, b_copy);
        }
        issued[0] = k;
    } else if (warp >= 1 && warp <= TC_ISSUERS && lane == 0) {
        /* the MMA issuers: issuer i takes stages i, i + TC_ISSUERS, ... into its own accumulator (8 Q columns at
         * 8 Q i), each stage's MMAs as soon as its copies have landed; a commit frees the stage for the producer. A
         * lone thread spends most of a stage issuing its MMAs, so several threads shorten the tile's chain. */
        const int ia = warp - 1;
        const uint32_t acc = tmem + (uint32_t)(8 * Q * ia);
        int last = -1;
        for (int k = ia; k < nk; k += TC_ISSUERS) {
            const int s = k % TC_STAGES;
            if (!mbar_wait(full0 + 8 * s, (uint32_t)((k / TC_STAGES) & 1))) {
                good = 0;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            /* K chunk kc starts 32 bytes further into the row and 2 Q core matrices further into the band block: the
             * descriptors' start fields (16-byte units, no carry below 256 KB) step by 2 and by 16 Q */
            const uint32_t a0 = smem_u32(smem + s * stage_bytes), b0 = a0 + a_bytes;
            const uint64_t ad = mdesc(a0, 16, 128), bd = mdesc(b0, Q * 128, 128);
            for (int kc = 0; kc < kchunks; kc++)
                tc_mma(acc, ad + 2u * kc, bd + (uint64_t)(16 * Q) * kc, idesc, (k != ia || kc != 0) ? 1u : 0u);
            tc_commit(empty0 + 8 * s);
            last = k;
        }
        issued[1 + ia] = last + 1;
        /* an issuer's last commit covers every MMA it issued */
        if (good && last >= 0)
            good = mbar_wait(empty0 + 8 * (last % TC_STAGES), (uint32_t)((last / TC_STAGES) & 1)) ? 1 : 0;
    }
    const int ok_all = __syncthreads_and(good);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!ok_all) {
        /* A wait gave up. Before the CTA frees its tensor memory and exits, what it started must be done: the MMAs of
         * every committed stage (the last commit tracks them all) and the bulk copies of every stage filled but not
         * consumed (each completes its full barrier's phase), else they would still write into tensor and shared
         * memory that the next CTA on this SM may own. These waits are bounded too; past them the engines themselves
         * have stopped and the context cannot be saved from here. */
        if (tid == 0) {
            atomicExch(err, 1);
            const int kp = issued[0];
            for (int i = 0; i < TC_ISSUERS; i++) {
                const int lk = issued[1 + i] - 1;
                if (lk >= 0)
                    mbar_wait(empty0 + 8 * (lk % TC_STAGES), (uint32_t)((lk / TC_STAGES) & 1));
            }
            /* a stage not committed by its issuer was not refilled: its barrier is still in that stage's phase */
            for (int k = 0; k < kp; k++)
                if (k >= issued[1 + k % TC_ISSUERS])
                    mbar_wait(full0 + 8 * (k % TC_STAGES), (uint32_t)((k / TC_STAGES) & 1));
        }
    } else {
        /* epilogue. The step is a power of two dividing the cell, and X0 - x0 is a multiple of 16, so the corner (x, y)
         * is on the step grid when (8 m + s) and y - y0 are multiples of it. */
        const int sh = __ffs(p.step) - 1;
        const int per = NCC_CELL >> sh;
        const int ly0 = (ty % (NCC_CELL / Q)) * Q; /* this tile's first row inside its cell row */
        uint32_t xmask = 0;
#pragma unroll
        for (int s = 0; s < 8; s++)
            if (xr + s <= p.x1 - p.x0 && ((8 * m + s) & (p.step - 1)) == 0)
                xmask |= 1u << s;
        float best = -2.0f;
        int bkey = 1 << 30;
#pragma unroll
        for (int cc = 0; cc < CH; cc++) {
            const int c = c0 + cc;
            /* columns 16 c .. 16 c + 15 (y-corners 2 c, 2 c + 1) of every issuer's accumulator, summed in issuer order */
            float v[16];
            {
                const uint32_t row = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(16 * c);
                uint32_t r[TC_ISSUERS][16];
#pragma unroll
                for (int i = 0; i < TC_ISSUERS; i++)
                    tc_ld16(row + (uint32_t)(8 * Q * i), r[i]);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int e = 0; e < 16; e++) {
                    v[e] = __uint_as_float(r[0][e]);
#pragma unroll
                    for (int i = 1; i < TC_ISSUERS; i++)
                        if (i < nk) /* an issuer with no stage left its accumulator unwritten */
                            v[e] += __uint_as_float(r[i][e]);
                }
            }
#pragma unroll
            for (int qq = 0; qq < 2; qq++) {
                const int q = 2 * c + qq, yr = ty * Q + q;
                if (yr >= fh || (yr & (p.step - 1)))
                    continue;
                const int i = 2 * cc + qq;
                const uint32_t jw[4] = {jr[i].x, jr[i].y, jr[i].z, jr[i].w};
                const float fq[8] = {fr[2 * i].x, fr[2 * i].y, fr[2 * i].z, fr[2 * i].w,
                                     fr[2 * i + 1].x, fr[2 * i + 1].y, fr[2 * i + 1].z, fr[2 * i + 1].w};
#pragma unroll
                for (int s = 0; s < 8; s++) {
                    if (!((xmask >> s) & 1u))
                        continue;
                    const float j0 = from16((uint16_t)(jw[s >> 1] >> (16 * (s & 1))), KIND);
                    /* a near-blank window's factor is 0: + 0 makes its score +0 whatever the sign of the sum, the
                     * reference's 0 (a -0 would order below the other cells' +0 in the top-8 keys) */
                    const float score = (v[8 * qq + s] - j0 * p.sum_t) * fq[s] + 0.0f;
                    const int key = ((ly0 + q) >> sh) * per + ((8 * (m & 1) + s) >> sh);
                    if (score > best || (score == best && key < bkey)) {
                        best = score;
                        bkey = key;
                    }
                }
            }
        }
        const float ob = __shfl_xor_sync(VTG_FULL, best, 1);
        const int okey = __shfl_xor_sync(VTG_FULL, bkey, 1);
        if (ob > best || (ob == best && okey < bkey)) {
            best = ob;
            bkey = okey;
        }
        const int ccol = tx * (TC_XS / NCC_CELL) + (m >> 1), crow = (Y0 - p.y0) / NCC_CELL;
        if ((m & 1) == 0 && ccol < p.ccols && crow < p.crows && bkey < (1 << 30))
            atomicMax(cellw + (size_t)crow * p.ccols + ccol, cell_word(best, bkey));
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tc_cols(Q)) : "memory");
    }
}

cudaError_t vtg_launch_ncc_map_tc(const void *plane, int pitch, int elem_bytes, const NccPrm &p, const NccScratch &s,
                                  int kind, cudaStream_t st)
{
    if (elem_bytes != 1 || !s.band || !s.conv || !s.fac || !s.cellw || (kind != VTG_NCC_BF16 && kind != VTG_NCC_FP16) ||
        p.tw > 128)
        return cudaErrorInvalidValue;
    const int krow = tc_krow(p.tw), q = tc_q(p.tw, p.th);
    const TcSmem sm = tc_smem(krow, q);
    const int fw = p.x1 - p.x0 + 1, fh = p.y1 - p.y0 + 1;
    const int tiles_x = (fw + TC_XS - 1) / TC_XS, tiles_y = (fh + q - 1) / q;
    const int cpitch = tiles_x * TC_XS + TC_MAX_KROW;
    const int fpitch = tiles_x * TC_XS; /* every tile's 1,024 corners inside a factor row */
    const int rows = p.y0 + tiles_y * q + p.th; /* every row a tile's band reads */
    if ((size_t)cpitch * rows > s.conv_elems || (size_t)fpitch * fh > s.fac_elems || (p.step & (p.step - 1)) ||
        NCC_CELL % p.step)
        return cudaErrorInvalidValue;
    const int cells = p.ccols * p.crows;
    cudaError_t e = cudaSuccess;
    const int btx = bp_tx(p.tw), bgx = (fw + btx - 1) / btx, nbox = bgx * ((fh + BP_TY - 1) / BP_TY);
    const int cgx = (cpitch / 8 + 255) / 256, nconv = cgx * rows;
    if ((long long)nconv * 256 < cells) /* the converting CTAs zero the cells' words */
        return cudaErrorInvalidValue;
    if (kind == VTG_NCC_BF16)
        ncc_prep<VTG_NCC_BF16><<<nbox + nconv, 256, 0, st>>>((const uint8_t *)plane, pitch, p, fw, fpitch, btx, bgx, nbox,
                                                             s.fac, rows, cpitch, cgx, s.conv, s.cellw, cells);
    else
        ncc_prep<VTG_NCC_FP16><<<nbox + nconv, 256, 0, st>>>((const uint8_t *)plane, pitch, p, fw, fpitch, btx, bgx, nbox,
                                                             s.fac, rows, cpitch, cgx, s.conv, s.cellw, cells);
    /* the map and the passes after it start as programmatic dependents (their launch and setup overlap the kernel
     * before), except when events around the map time it alone */
    const bool pdl = !s.map_ev0;
#define MAP_TC(K, QQ)                                                                                                  \
    do {                                                                                                               \
        e = cudaFuncSetAttribute(ncc_map_tc<K, QQ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm.total);       \
        if (e != cudaSuccess)                                                                                          \
            return e;                                                                                                  \
        if (s.map_ev0 && (e = cudaEventRecord(s.map_ev0, st)) != cudaSuccess)                                          \
            return e;                                                                                                  \
        e = vtg_launch_k(ncc_map_tc<K, QQ>, dim3(tiles_x * tiles_y), dim3(TcShape<QQ>::threads), sm.total, st, pdl,    \
                         p, (const uint16_t *)s.band, krow, tiles_x, sm.a_bytes, sm.stage_bytes,                        \
                         (const uint16_t *)s.conv, cpitch, (const float *)s.fac, fpitch, s.cellw, s.err);              \
        if (e != cudaSuccess)                                                                                          \
            return e;                                                                                                  \
        if (s.map_ev1 && (e = cudaEventRecord(s.map_ev1, st)) != cudaSuccess)                                          \
            return e;                                                                                                  \
    } while (0)
    if (kind == VTG_NCC_BF16) {
        if (q == 8)
            MAP_TC(VTG_NCC_BF16, 8);
        else
            MAP_TC(VTG_NCC_BF16, 16);
    } else {
        if (q == 8)
            MAP_TC(VTG_NCC_FP16, 8);
        else
            MAP_TC(VTG_NCC_FP16, 16);
    }
#undef MAP_TC
    if ((e = cudaGetLastError()) != cudaSuccess)
        return e;
    /* the cells from their words, and their best eight */
    return vtg_launch_ncc_top(p, s, true, st, pdl);
}
