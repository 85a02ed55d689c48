// dcpse_gram_tc.cuh -- the Gram products A = B^T B of the fast assembly on the
// fifth-generation tensor cores (tcgen05, bf16 operands, FP32 accumulators in
// tensor memory), from a 62-bit fixed-point representation of B.  Included by
// dcpse_assemble.cu: it builds B with that file's monomial program.
//
// B is the k x nu matrix of a particle's scaled monomials (Dcpse.hpp:745-757,
// B = E V), built in FP64 with the same operations as the SIMT Gram kernel by
// gram_b_kernel (one warp per particle, many per SM: the FP64 work needs the
// latency hiding), which stores it with the exponent E_j of each column's
// largest entry (|B_qj| < 2^E_j).  Here every entry becomes the integer
//     F = round(B_qj 2^(62 - E_j)),  |F| < 2^62,
// written as eight balanced digits of 8 bits,
//     F = sum_(a=0..7) d_a 2^(8 (7 - a)),  d_0 in [-64, 64], d_(a>0) in [-128, 127],
// each exact in bf16.  The digits sit in shared memory as a matrix of 8 nu
// rows (row 8 j + a = digit a of column j; K = neighbour q).  MMAs of 16
// neighbours, M = 128 (rows 0-127: columns i < 16, all digits) x N = 8 nu
// rounded to 16 (all columns j), put
//     P_ab(i, j) = sum_q d_a(q, i) d_b(q, j)
// in tensor-memory lane 8 i + a, column 8 j + b (a second set, rows 128-255
// against the columns j >= 16, serves i >= 16).  |d_a d_b| <= 2^14, so for
// k <= 128 every |P_ab| < 2^21 and the FP32 accumulation is exact.  The
// lanes leave the products of shifts a + b <= 7 in shared memory, and the
// entries' pass forms the shift sums S_s = sum_(a+b=s) P_ab (at most 8
// products: exact in FP32) and
//     H = sum_(s<=3) S_s 2^(8 (3 - s)),  L = sum_(s=4..7) S_s 2^(8 (7 - s))
// in 64-bit integers (shifts s >= 8 are dropped, below 2^-58 of
// 2^(E_i + E_j)), so that
//     sum_q F_qi F_qj = 2^56 (H 2^32 + L) + (dropped shifts).
// The entry is the FP64 rounding of 2^56 (H 2^32 + L) times 2^(E_i + E_j - 124):
// about as accurate as a correctly rounded Gram entry relative to the
// columns' scales, more accurate than a sequential FP64 sum, and not
// bit-identical to the reference order (which the SIMT Gram kernel keeps).
//
// One CTA of 24 warps per SM, as a pipeline:
//   two digit groups g = 0, 1 (warps 8 g .. 8 g + 7) take every other
//     particle of the CTA's share; a neighbour and half the columns per
//     thread; the digits into
//     stack[g]; the group's thread 0 then issues the particle's MMAs into
//     accumulator[g] and commits them to mma_done[g];
//   the epilogue (warps 16-23; warps 16 + w and 20 + w read lanes 32 w ..
//     32 w + 31, alternate batches of four columns j) takes the groups'
//     particles in turn, moves the digit products of every pair (i <= j) to
//     shared memory, four columns j per tensor-memory load,
//     frees the accumulator (acc_free[g]) and turns the products into
//     entries.
// Every wait on an mbarrier is bounded; one that runs out raises the CTA's
// abort flag, which ends all loops.
//
// Shared-memory layout of a stack: the canonical K-major layout without
// swizzle (core matrices of 8 rows x 16 bytes; the core matrix of column j
// holds its eight digits), the next core matrix along K 144 bytes on (LBO:
// 128 bytes plus 16 of skew, so that the 2-byte stores of a warp's 32
// neighbours fall on 16 distinct banks), the next 8-row group kc / 8 * 144
// bytes on (SBO).

constexpr int kTcGroup = 256;          // threads of a digit group: a neighbour and half the columns each
constexpr int kTcEpi = 256;            // threads of the epilogue: two warps per lane quarter
constexpr int kTcThreads = 2 * kTcGroup + kTcEpi;
constexpr int kTcMaxK = 128;           // neighbours of one pass
constexpr int kTcMaxNu = 24;           // the two accumulators' columns fit in 256
constexpr uint32_t kTcLbo = 144;       // bytes between core matrices along K
constexpr uint32_t kTcAccCols = 256;   // tensor-memory columns of a group's products
constexpr long kTcWaitLimit = 1L << 24;  // polls of an mbarrier before giving up

struct TcLayout {
    int kc;                 // K extent of the planes (multiple of 16, <= kTcMaxK)
    uint32_t sbo;           // bytes between 8-row groups
    uint32_t stack_bytes;   // one stack: 32 row groups (256 rows)
    uint32_t sum_off;       // the digit products of the pairs, [a][b][pstride] floats
    int pstride;            // npairs rounded up to 32, plus 1 (bank skew)
    uint32_t bytes;         // dynamic shared memory of the CTA
};

// Shared memory of a CTA for planes of up to maxk neighbours and npairs Gram
// entries.
inline TcLayout tc_layout(int maxk, int npairs) {
    TcLayout L{};
    L.kc = ((std::max(maxk, 1) + 15) / 16) * 16;
    L.sbo = (uint32_t)(L.kc / 8) * kTcLbo;
    L.stack_bytes = 32u * L.sbo;
    L.sum_off = 2u * L.stack_bytes;
    L.pstride = ((std::max(npairs, 1) + 31) / 32) * 32 + 1;
    L.bytes = L.sum_off + 64u * (uint32_t)L.pstride * (uint32_t)sizeof(float);
    // more than half of an SM's shared memory: a second CTA, which would wait
    // for the tensor memory of the first, cannot be placed beside it
    L.bytes = std::max(L.bytes, 120u * 1024u);
    return L;
}

// what a digit group hands to the epilogue with a particle's products
struct TcMeta {
    int64_t slot;  // batch slot; -1: no more particles
    int E[32];     // column exponents
};

__device__ __forceinline__ uint32_t tc_smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start >> 4 (bits 0-13), LBO >> 4 (16-29),
// SBO >> 4 (32-45), descriptor version 1 (bits 46-47), base offset 0, no
// swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((kTcLbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A and B bf16
// (bits 7-9 and 10-12 = 1), both K-major (bits 15, 16 = 0), N (bits 17-22 =
// N >> 3; N a multiple of 16 up to 256), M = 128 (bits 24-28 = M >> 4)
__host__ __device__ constexpr uint32_t tc_idesc(uint32_t n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t da, uint64_t db, uint32_t idesc,
                                       uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(da), "l"(db), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_bar(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

__device__ __forceinline__ void tc_mbar_init(uint64_t* m, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc_smem_u32(m)), "r"(count) : "memory");
}
__device__ __forceinline__ void tc_mbar_arrive(uint64_t* m) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc_smem_u32(m)) : "memory");
}

// Waits (bounded) for the completion of the phase of parity `parity`; gives
// up when the CTA's abort flag is raised or the polls run out (raising it).
__device__ bool tc_mbar_wait(uint64_t* m, uint32_t parity, volatile int* abort_flag) {
    for (long it = 0; it < kTcWaitLimit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(tc_smem_u32(m)), "r"(parity)
            : "memory");
        if (done) return true;
        if (*abort_flag) return false;
    }
    *abort_flag = 1;
    return false;
}

__device__ __forceinline__ void tc_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// round(x 2^(62 - E)) for |x| < 2^E, from the double's bits (integer pipe;
// selects, no branches: neighbours of a warp differ in their shifts)
__device__ __forceinline__ long long tc_fixed62(double x, int E) {
    const long long bits = __double_as_longlong(x);
    const int eb = (int)((bits >> 52) & 0x7ff);
    const unsigned long long m = (unsigned long long)(bits & 0xFFFFFFFFFFFFFll) | (1ull << 52);
    const int sh = eb - 1013 - E;  // x 2^(62 - E) = m 2^sh, sh <= 9 since |x| < 2^E
    const int rs = min(max(-sh, 1), 63);
    const unsigned long long up = m << max(sh, 0);
    const unsigned long long down = (m + (1ull << (rs - 1))) >> rs;
    unsigned long long F = sh >= 0 ? up : down;
    F = (eb == 0 || sh <= -63) ? 0ull : F;  // zero, subnormals and values below the precision
    return bits < 0 ? -(long long)F : (long long)F;
}

// bf16 bits of a signed byte of w (exact: at most 8 significant bits); the
// float of the byte by the 1.5 * 2^23 offset (integer and FP32 adds)
__device__ __forceinline__ unsigned short tc_bf16_of_byte(unsigned w, int byte) {
    const int d = (int)(signed char)(w >> (8 * byte));
    const float f = __int_as_float(0x4B400000 + d) - 12582912.0f;
    return (unsigned short)(__float_as_uint(f) >> 16);
}


// The Gram entries of the particles [b0, b1) of a batch from their B
// (S.bmat, S.bexp): CTA c, group g takes the particles b0 + (2 c + g) +
// 2 t gridDim.x, t = 0, 1, ...
__global__ void __launch_bounds__(kTcThreads, 1)
    gram_tc_kernel(AsmArgs a, Split S, int64_t b0, int64_t b1, TcLayout L) {
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    __shared__ __align__(8) uint64_t mma_done[2];  // per group: the products' commit + the meta arrive
    __shared__ __align__(8) uint64_t acc_free[2];  // per group: one arrive per epilogue warp
    __shared__ __align__(8) uint64_t drain[2];     // per group: every product it issued is done
    __shared__ TcMeta meta[2];
    __shared__ uint32_t tmem_slot;
    __shared__ short pidx[kTcMaxNu][kTcMaxNu];  // pair (i <= j) -> Gram entry, -1 if not needed
    __shared__ int sEb[2][32], sEe[32];  // column exponents: the groups' current particles, the epilogue's
    __shared__ int b_go[2], e_go;        // uniform decisions of the groups and of the epilogue
    __shared__ volatile int abort_flag;
    const AsmTables& T = *a.tab;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nu = T.nu, npairs = T.npairs;
    // tensor-memory columns of the products of the rows i < 16 and i >= 16
    const uint32_t n1 = (uint32_t)((8 * nu + 15) & ~15), n2 = nu > 16 ? (uint32_t)((8 * (nu - 16) + 15) & ~15) : 0u;
    float* prod = reinterpret_cast<float*>(tc_smem + L.sum_off);  // P_ab of pair e at (8 a + b) pstride + e
    const int ps = L.pstride;

    // rows 8 nu .. 255 of both stacks stay zero for the whole kernel
    for (uint32_t i = tid; i < 2u * L.stack_bytes / 16u; i += kTcThreads)
        reinterpret_cast<uint4*>(tc_smem)[i] = make_uint4(0u, 0u, 0u, 0u);
    for (int i = tid; i < kTcMaxNu * kTcMaxNu; i += kTcThreads) (&pidx[0][0])[i] = -1;
    if (tid == 0) {
        for (int g = 0; g < 2; ++g) {
            tc_mbar_init(&mma_done[g], 2);
            tc_mbar_init(&acc_free[g], kTcEpi / 32);
            tc_mbar_init(&drain[g], 1);
        }
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         tc_smem_u32(&tmem_slot)),
                     "r"(2u * kTcAccCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    __syncthreads();
    for (int e = tid; e < npairs; e += kTcThreads) pidx[T.pi[e]][T.pj[e]] = (short)e;
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;

    if (tid < 2 * kTcGroup) {
        // -------------------------------------------------- digit group g --
        const int g = tid / kTcGroup, gtid = tid % kTcGroup;
        const int j_lo = (gtid >> 7) * (kTcMaxNu / 2);  // this thread's half of the columns
        const int bar_id = 1 + g;
        unsigned char* stack = tc_smem + (uint32_t)g * L.stack_bytes;
        const uint32_t acc = tmem + (uint32_t)g * kTcAccCols;
        const int ngroups = T.ngroups;
        const int q = gtid & 127;  // this thread's neighbour
        unsigned char* col = stack + (uint32_t)(q >> 3) * kTcLbo + (uint32_t)(q & 7) * 2u;
        int n = 0;           // particles handed to the epilogue
        for (int64_t it = b0 + 2 * (int64_t)blockIdx.x + g;; it += 2 * (int64_t)gridDim.x) {
            // completion n - 1 of the group's barriers: its previous particle
            // (parity 1 before the first: already complete)
            const uint32_t prev = ((uint32_t)n & 1u) ^ 1u;
            if (it >= b1) {
                // no more particles: a terminal meta for the epilogue
                if (gtid == 0 && tc_mbar_wait(&acc_free[g], prev, &abort_flag) &&
                    tc_mbar_wait(&mma_done[g], prev, &abort_flag)) {
                    meta[g].slot = -1;
                    tc_mbar_arrive(&mma_done[g]);
                    tc_mbar_arrive(&mma_done[g]);
                }
                break;
            }
            const int64_t slot = it - b0;
            const int32_t word = S.gst[slot];
            bool any_ok = false;
            for (int gr = 0; gr < ngroups; ++gr) any_ok |= group_status(word, gr) == ST_OK;
            if (!any_ok) continue;  // not assembled: its Gram entries are not read
            const int64_t p = a.order ? (int64_t)a.order[it] : it;
            const int k = (int)(a.rowptr[p + 1] - a.rowptr[p]);  // <= kTcMaxK (checked by the host)
            const int kq = (k + 15) & ~15;
            // this thread's row of B (zeros for the columns k .. kq - 1 of the last MMA)
            const double* Bq = S.bmat + slot * (int64_t)nu * S.kpad + q;
            double bq[kTcMaxNu / 2];
#pragma unroll
            for (int jj = 0; jj < kTcMaxNu / 2; ++jj)
                if (j_lo + jj < nu) bq[jj] = q < k ? Bq[(int64_t)(j_lo + jj) * S.kpad] : 0.0;
            if (gtid < 32) sEb[g][gtid] = S.bexp[slot * 32 + gtid];
            // the stack is free once the group's previous products are done
            if (gtid == 0) b_go[g] = tc_mbar_wait(&mma_done[g], prev, &abort_flag) ? 1 : 0;
            tc_bar(bar_id, kTcGroup);
            if (!b_go[g]) break;

            // the eight digits of column j into rows 8 j .. 8 j + 7 (one core
            // matrix; row 8 j + a holds byte 7 - a of X)
            if (q < kq) {
#pragma unroll
                for (int jj = 0; jj < kTcMaxNu / 2; ++jj) {
                    const int j = j_lo + jj;
                    if (j < nu) {
                        const unsigned long long X =
                            (unsigned long long)(tc_fixed62(bq[jj], sEb[g][j]) + 0x0080808080808080ll) ^
                            0x0080808080808080ull;
                        const unsigned xl = (unsigned)X, xh = (unsigned)(X >> 32);
                        unsigned char* cm = col + (uint32_t)j * L.sbo;
                        *reinterpret_cast<unsigned short*>(cm) = tc_bf16_of_byte(xh, 3);
                        *reinterpret_cast<unsigned short*>(cm + 16) = tc_bf16_of_byte(xh, 2);
                        *reinterpret_cast<unsigned short*>(cm + 32) = tc_bf16_of_byte(xh, 1);
                        *reinterpret_cast<unsigned short*>(cm + 48) = tc_bf16_of_byte(xh, 0);
                        *reinterpret_cast<unsigned short*>(cm + 64) = tc_bf16_of_byte(xl, 3);
                        *reinterpret_cast<unsigned short*>(cm + 80) = tc_bf16_of_byte(xl, 2);
                        *reinterpret_cast<unsigned short*>(cm + 96) = tc_bf16_of_byte(xl, 1);
                        *reinterpret_cast<unsigned short*>(cm + 112) = tc_bf16_of_byte(xl, 0);
                    }
                }
            }
            // the planes become visible to the tensor cores (async proxy)
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            tc_fence_before();
            tc_bar(bar_id, kTcGroup);
            // the MMAs of 16 neighbours, once the epilogue has read the
            // group's accumulator and meta of its previous particle
            if (gtid == 0 && tc_mbar_wait(&acc_free[g], prev, &abort_flag)) {
                tc_fence_after();
                meta[g].slot = slot;
#pragma unroll
                for (int j = 0; j < 32; ++j) meta[g].E[j] = S.bexp[slot * 32 + j];  // the group may rewrite sEb
                const uint32_t base = tc_smem_u32(stack), hi_rows = 16u * L.sbo;
                for (int t = 0; t < kq / 16; ++t) {
                    const uint32_t ko = (uint32_t)t * 2u * kTcLbo;
                    const uint64_t d1 = tc_desc(base + ko, L.sbo);
                    tc_mma(acc, d1, d1, tc_idesc(n1), t > 0 ? 1u : 0u);
                    if (n2) {
                        const uint64_t d2 = tc_desc(base + hi_rows + ko, L.sbo);
                        tc_mma(acc + n1, d2, d2, tc_idesc(n2), t > 0 ? 1u : 0u);
                    }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 tc_smem_u32(&mma_done[g]))
                             : "memory");
                tc_mbar_arrive(&mma_done[g]);  // release: the meta is seen with the products
            }
            ++n;
        }
        // every product issued by this group completes before the columns are freed
        if (gtid == 0) {
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             tc_smem_u32(&drain[g]))
                         : "memory");
            volatile int no_abort = 0;
            tc_mbar_wait(&drain[g], 0u, &no_abort);
        }
    } else {
        // ------------------------------------------------------ epilogue --
        const int etid = tid - 2 * kTcGroup;
        const int ew = (etid >> 5) & 3;  // this warp reads lanes 32 ew .. 32 ew + 31,
        const int part = etid >> 7;      // every other batch of four columns
        const int da = lane & 7;   // digit a of the A row; row i = 4 ew + lane / 8 (+ 16)
        const int i1 = 4 * ew + (lane >> 3);
        const uint32_t lanes = (uint32_t)(ew * 32) << 16;
        float* prow = prod + 8 * da * ps;  // this lane's products P_ab, b = 0..7
        int use[2] = {0, 0};
        bool done[2] = {false, false};
        for (int g = 0; !(done[0] && done[1]); g ^= 1) {
            if (done[g]) continue;
            if (etid == 0) e_go = tc_mbar_wait(&mma_done[g], (uint32_t)use[g] & 1u, &abort_flag) ? 1 : 0;
            tc_bar(3, kTcEpi);
            if (!e_go) break;
            ++use[g];
            const int64_t slot = meta[g].slot;
            if (slot < 0) {
                done[g] = true;
                continue;
            }
            if (etid < 32) sEe[etid] = meta[g].E[etid];
            tc_fence_after();
            // pair (i, j), i <= j: lane (i, a) stores P_ab(i, j), a + b <= 7;
            // four columns j per load
            // (columns 8 j .. 8 j + 31 of the group's 256 stay inside them
            // for nu <= 24)
            const uint32_t acc = tmem + (uint32_t)g * kTcAccCols + lanes;
#pragma unroll 1
            // the quarter's batches of both row blocks alternate between its two warps
            int batch = 0;
            for (int half = 0; half < 2; ++half) {
                if (half && !n2) break;
                const int i = i1 + 16 * half, j0 = 4 * ew + 16 * half;
                const uint32_t c0 = half ? n1 : 0u;
                for (int jb = j0; jb < nu; jb += 4) {  // warp-uniform: from the quarter's smallest i
                    if ((batch++ & 1) != part) continue;
                    uint32_t r[32];
                    tc_ld32(acc + c0 + (uint32_t)(8 * (jb - 16 * half)), r);
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        // the products of shifts a + b <= 7 for the entries' pass
                        const int j = jb + u;
                        const int e = (i <= j && j < nu) ? pidx[i][j] : -1;
                        if (e >= 0) {
#pragma unroll
                            for (int b = 0; b < 8; ++b)
                                if (da + b <= 7) prow[b * ps + e] = __uint_as_float(r[8 * u + b]);
                        }
                    }
                }
            }
            // the accumulator and the meta are free for the group's next particle
            tc_fence_before();
            __syncwarp();
            if (lane == 0) tc_mbar_arrive(&acc_free[g]);
            tc_bar(3, kTcEpi);
            // the entries: the shift sums S_s = sum_(a+b=s) P_ab (exact in FP32:
            // at most 8 products below 2^21), H and L in 64-bit integers, one
            // rounding of 2^56 (H 2^32 + L) and the columns' scales
            // 2^(E_i - 62) 2^(E_j - 62)
            for (int e = etid; e < npairs; e += kTcEpi) {
                const int pi = T.pi[e], pj = T.pj[e];
                long long H = 0, Lo = 0;
#pragma unroll
                for (int sh = 0; sh < 8; ++sh) {
                    float sum = 0.0f;
#pragma unroll
                    for (int a0 = 0; a0 <= sh; ++a0) sum += prod[(8 * a0 + sh - a0) * ps + e];
                    const long long v = (long long)__float2int_rn(sum);
                    if (sh <= 3)
                        H += v * (1ll << (8 * (3 - sh)));
                    else
                        Lo += v * (1ll << (8 * (7 - sh)));
                }
                const double v = fma((double)H, 4294967296.0 /* 2^32 */, (double)Lo);
                S.gram[slot * S.gstride + e] =
                    (v * pow2i(max(sEe[pi] - 34, -1022))) * pow2i(max(sEe[pj] - 34, -1022));
            }
            tc_bar(3, kTcEpi);  // sums and exponents are rewritten by the next particle
        }
    }
    if (abort_flag && tid == 0) atomicExch(a.err, 1);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2u * kTcAccCols)
                     : "memory");
}
