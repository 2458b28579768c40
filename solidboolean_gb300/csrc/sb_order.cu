// The reference's processing orders, reproduced with data-parallel kernels.
//
// Iteration order of a libstdc++ unordered container (identity hash, max load factor 1, unique keys,
// single-element inserts) as a function of the insertion sequence, stage by stage. A stage holds one
// bucket count B (13, 29, 59, ...: the element count at which the table grows, hash_bucket_count) and
// covers the inserts made while the table has that count. Within it:
//   * the growth at its start rebuilds the list by walking the old list and putting each node at the front
//     of its bucket's run, or, when its bucket is still empty, at the front of the list; so runs are ordered
//     by the old position of their first node, latest first, and each run holds its nodes latest first;
//   * an insert into a non-empty bucket goes to the front of that bucket's run, an insert into an empty one
//     opens a run at the front of the list.
// So at the end of a stage every node's position is a rank by one composite key: runs opened by this
// stage's inserts first (latest opened first), then the rebuilt runs (in rebuilt order); inside a run this
// stage's inserts first (latest first), then the rebuilt nodes (in rebuilt order). One block computes the
// ranks of all stages: a scatter into buckets, a count per run, a scan, and a short walk of each bucket.
//
// The reference tree's traversal order of a candidate pair (src/axisalignedboundingboxtree.h:54-88): the
// dual descent goes from the two roots, descending the first tree when the second node is a leaf or when
// the first node has at least as many members, else the second, left child first; at two leaves it lists
// the first leaf's members, each against the second leaf's members. The bits of the descent path (left-
// aligned), then the two positions inside the leaves, order pairs as the traversal emits them.
#include <algorithm>
#include <climits>
#include <mutex>

#include "sb_ktime.h"
#include "sb_order.cuh"

namespace sbg {

constexpr int kOrderThreads = 1024;
constexpr int kPathBits = 53; // key: mesh bit, 53 path bits, 5 + 5 bits of leaf positions (leaves hold <= 20)

// ---------------------------------------------------------------------------------------------------
// block-wide helpers (every thread of the block calls them)
// ---------------------------------------------------------------------------------------------------

// in-place exclusive scan of a[0..n) (global memory); returns the total
__device__ int block_excl_scan(int *a, int n)
{
    __shared__ int warpTot[32];
    __shared__ int total;
    const int T = blockDim.x, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int per = (n + T - 1) / T;
    const int b0 = min(n, tid * per), b1 = min(n, b0 + per);
    int local = 0;
    for (int i = b0; i < b1; ++i)
        local += a[i];
    int incl = local;
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o)
            incl += v;
    }
    if (lane == 31)
        warpTot[w] = incl;
    __syncthreads();
    if (w == 0) {
        const int x = lane < (T >> 5) ? warpTot[lane] : 0;
        int y = x;
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xFFFFFFFFu, y, o);
            if (lane >= o)
                y += v;
        }
        warpTot[lane] = y - x;
        if (lane == 31)
            total = y;
    }
    __syncthreads();
    int run = warpTot[w] + incl - local;
    for (int i = b0; i < b1; ++i) {
        const int v = a[i];
        a[i] = run;
        run += v;
    }
    const int tot = total;
    __syncthreads();
    return tot;
}

size_t hash_scratch_ints(int n)
{
    const size_t N = (size_t)std::max(n, 1);
    return 6 * N + 1 + 2 * (size_t)hash_bucket_count((uint32_t)N) + 8;
}

HashScratch hash_scratch_at(int *base, int n)
{
    const size_t N = (size_t)std::max(n, 1);
    const size_t B = hash_bucket_count((uint32_t)N);
    HashScratch h;
    h.posA = base;
    h.posB = h.posA + N;
    h.slotOf = h.posB + N;
    h.nxt = h.slotOf + N;
    h.runSize = h.nxt + N;
    h.bmin = h.runSize + 2 * N + 1;
    h.head = h.bmin + B;
    return h;
}

// One stage: M elements (the first Mprev of them placed by the previous stage at pos[]) in B buckets ->
// npos[]. Per bucket, the smallest of (old element: its old position; new element i: Mprev + i) tells both
// whether the bucket holds old elements and the run's key. bkt[] keeps each element's bucket for the stage.
__device__ void hash_stage(const uint32_t *keys, int M, int Mprev, uint32_t B, const int *pos, int *npos,
                           int *bkt, int *nxt, int *runSize, int *bmin, int *head)
{
    const int T = blockDim.x, tid = threadIdx.x;
    for (uint32_t b = tid; b < B; b += T) {
        bmin[b] = INT_MAX;
        head[b] = -1;
    }
    for (int i = tid; i < M + Mprev; i += T)
        runSize[i] = 0;
    __syncthreads();
    for (int i = tid; i < M; i += T) {
        const int b = (int)(keys[i] % B);
        bkt[i] = b;
        atomicMin(&bmin[b], i < Mprev ? pos[i] : Mprev + i);
        nxt[i] = atomicExch(&head[b], i);
    }
    __syncthreads();
    // runs: opened by this stage's inserts [0, M - Mprev), latest first; rebuilt [M, M + Mprev)
    for (int i = tid; i < M; i += T) {
        const int v = bmin[bkt[i]];
        atomicAdd(&runSize[v < Mprev ? M + (Mprev - 1 - v) : (M - 1 - (v - Mprev))], 1);
    }
    __syncthreads();
    block_excl_scan(runSize, M + Mprev);
    for (int i = tid; i < M; i += T) {
        const int b = bkt[i];
        const int v = bmin[b];
        const int slot = v < Mprev ? M + (Mprev - 1 - v) : (M - 1 - (v - Mprev));
        const int gi = i < Mprev ? 1 : 0;
        const int ki = gi ? (Mprev - 1 - pos[i]) : (M - 1 - i);
        int within = 0;
        for (int j = head[b]; j >= 0; j = nxt[j]) {
            if (j == i)
                continue;
            const int gj = j < Mprev ? 1 : 0;
            const int kj = gj ? (Mprev - 1 - pos[j]) : (M - 1 - j);
            within += (gj < gi || (gj == gi && kj < ki)) ? 1 : 0;
        }
        npos[i] = runSize[slot] + within;
    }
    __syncthreads();
}

// keys[i]: the i-th inserted key (distinct); out[i]: its position in the container's iteration order. The
// keys and the stages whose arrays fit in smem (smemInts ints of shared memory) run there; the later stages
// in w.
__device__ void hash_order_block(const uint32_t *keysIn, int n, int *out, HashScratch w, int *smem, int smemInts)
{
    const int T = blockDim.x, tid = threadIdx.x;
    if (n <= 0)
        return;
    // keys cached in shared memory when they fit with room to spare
    const bool keysS = 2ll * n <= (long long)smemInts;
    const uint32_t *keys = keysIn;
    if (keysS) {
        uint32_t *k = reinterpret_cast<uint32_t *>(smem);
        for (int i = tid; i < n; i += T)
            k[i] = keysIn[i];
        keys = k;
        smem += (n + 3) & ~3;
        smemInts -= (n + 3) & ~3;
        __syncthreads();
    }
    // the largest stage whose arrays fit: two position buffers, buckets, links, runs (2 M + 1), 2 B per bucket
    int capM = 0;
    uint32_t capB = 0;
    {
        int mp = 0;
        for (int st = 0; st < 64; ++st) {
            const uint32_t Bs = hash_bucket_count((uint32_t)mp + 1);
            const int Ms = (uint32_t)n < Bs ? n : (int)Bs;
            if (6ll * Ms + 1 + 2ll * Bs > (long long)smemInts)
                break;
            capM = Ms;
            capB = Bs;
            mp = Ms;
            if (Ms == n)
                break;
        }
    }
    int *S0 = smem, *S1 = S0 + capM, *sBkt = S1 + capM, *sNxt = sBkt + capM, *sRun = sNxt + capM;
    int *sBmin = sRun + 2 * capM + 1, *sHead = sBmin + capB;
    bool inS = capM > 0;
    int *pos = inS ? S0 : w.posA, *npos = inS ? S1 : w.posB;
    int Mprev = 0;
    for (int stage = 0; stage < 64; ++stage) {
        const uint32_t B = hash_bucket_count((uint32_t)Mprev + 1);
        const int M = (uint32_t)n < B ? n : (int)B;
        if (inS && M > capM) {
            // leave shared memory: the previous stage's positions move to the global buffers
            for (int i = tid; i < Mprev; i += T)
                w.posA[i] = pos[i];
            __syncthreads();
            inS = false;
            pos = w.posA;
            npos = w.posB;
        }
        if (inS)
            hash_stage(keys, M, Mprev, B, pos, npos, sBkt, sNxt, sRun, sBmin, sHead);
        else
            hash_stage(keys, M, Mprev, B, pos, npos, w.slotOf, w.nxt, w.runSize, w.bmin, w.head);
        int *t = pos;
        pos = npos;
        npos = t;
        Mprev = M;
        if (M == n)
            break;
    }
    for (int i = tid; i < n; i += T)
        out[i] = pos[i];
    __syncthreads();
}

// ---------------------------------------------------------------------------------------------------
// cut faces: traversal key of the first pair, then the context map's iteration order
// ---------------------------------------------------------------------------------------------------

// The first pair of a face in the traversal: a first-mesh face meets second-mesh leaves left to right (a split
// of the first tree never reorders the second), so its first pair is the one with the smallest second-mesh leaf
// position, which is where the face's pair list starts; likewise for second-mesh faces.
__global__ void k_face_keys(FaceOrderArgs a)
{
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= a.nFaces)
        return;
    const unsigned long long side = f >= a.FA ? 1ull : 0ull;
    a.val[f] = f;
    if (!a.exact) {
        a.key[f] = (side << 63) | (unsigned long long)(unsigned)a.faceTri[f];
        return;
    }
    const int j = a.pairIdx[a.faceBegin[f]];
    const int ta = (int)a.pairAB[2 * (size_t)j], tb = (int)a.pairAB[2 * (size_t)j + 1];
    const int ra = a.A.rank[ta], rb = a.B.rank[tb];
    int4 na = a.A.tnode[0], nb = a.B.tnode[0];
    unsigned long long path = 0;
    int len = 0;
    bool bad = false;
    for (int step = 0; step < 4096; ++step) {
        // a child id outside the table (a failed build, reported by its own status) ends the walk
        if (na.z >= 0 && (na.z + 1 >= a.A.tnodeCount))
            na.z = -1, bad = true;
        if (nb.z >= 0 && (nb.z + 1 >= a.B.tnodeCount))
            nb.z = -1, bad = true;
        const bool leafA = na.z < 0, leafB = nb.z < 0;
        if (leafA && leafB)
            break;
        const bool descendB = leafA || (!leafB && na.y < nb.y);
        int bit;
        if (descendB) {
            const int4 l = a.B.tnode[nb.z];
            bit = rb >= l.x + l.y ? 1 : 0;
            nb = bit ? a.B.tnode[nb.z + 1] : l;
        } else {
            const int4 l = a.A.tnode[na.z];
            bit = ra >= l.x + l.y ? 1 : 0;
            na = bit ? a.A.tnode[na.z + 1] : l;
        }
        if (len < kPathBits)
            path = (path << 1) | (unsigned long long)bit;
        ++len;
    }
    if (len > kPathBits || bad) {
        atomicAdd(a.overflow, 1u);
        len = min(len, kPathBits);
    }
    const unsigned long long posA = (unsigned long long)max(0, min(ra - na.x, 31));
    const unsigned long long posB = (unsigned long long)max(0, min(rb - nb.x, 31));
    a.key[f] = (side << 63) | ((path << (kPathBits - len)) << 10) | (posA << 5) | posB;
}

// one block per mesh: the faces in insertion order (sorted by key) -> iteration order of the context map
constexpr int kCtxSortMax = 8192; // faces per mesh that k_face_ctx sorts in shared memory

// Bitonic sort of the mesh's faces by (key, face id) in shared memory (n <= kCtxSortMax); writes the face
// ids in order to out. Keys of one mesh's faces are distinct (distinct first pairs), the id only breaks ties
// that cannot occur.
__device__ void face_block_sort(const unsigned long long *key, const int *val, int n, int *out, int *smem)
{
    const int T = blockDim.x, tid = threadIdx.x;
    int N = 1;
    while (N < n)
        N <<= 1;
    unsigned long long *sk = reinterpret_cast<unsigned long long *>(smem);
    int *sv = reinterpret_cast<int *>(sk + N);
    for (int i = tid; i < N; i += T) {
        sk[i] = i < n ? key[i] : ~0ull;
        sv[i] = i < n ? val[i] : INT_MAX;
    }
    __syncthreads();
    for (int k = 2; k <= N; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = tid; i < N; i += T) {
                const int ixj = i ^ j;
                if (ixj <= i)
                    continue;
                const unsigned long long ka = sk[i], kb = sk[ixj];
                const int va = sv[i], vb = sv[ixj];
                const bool aAfter = ka > kb || (ka == kb && va > vb);
                if ((i & k) == 0 ? aAfter : !aAfter) {
                    sk[i] = kb;
                    sk[ixj] = ka;
                    sv[i] = vb;
                    sv[ixj] = va;
                }
            }
            __syncthreads();
        }
    for (int i = tid; i < n; i += T)
        out[i] = sv[i];
    __syncthreads();
}

__global__ void __launch_bounds__(kOrderThreads) k_face_ctx(FaceOrderArgs a, int smemInts)
{
    extern __shared__ __align__(16) int dsm[];
    const int side = blockIdx.x;
    const int off = side ? a.FA : 0, n = side ? a.FB : a.FA;
    if (a.blockSort)
        face_block_sort(a.key + off, a.val + off, n, a.sortedOut + off, dsm);
    uint32_t *keys = a.insKeys + off;
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        keys[i] = (uint32_t)a.faceTri[a.sortedVal[off + i]];
    __syncthreads();
    const HashScratch w = a.hs[side];
    // the result lands in slotOf, which the stages no longer need when it is written
    hash_order_block(keys, n, w.slotOf, w, dsm, smemInts);
    // the positions must be a permutation of [0, n); should they not be, the faces keep index order (and the
    // overflow counter reports it) rather than index out of bounds later
    __shared__ int bad;
    if (threadIdx.x == 0)
        bad = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        w.posA[i] = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int p = w.slotOf[i];
        if (p < 0 || p >= n || atomicAdd(&w.posA[p], 1) != 0)
            bad = 1;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int f = bad ? off + i : a.sortedVal[off + i];
        const int r = off + (bad ? i : w.slotOf[i]);
        a.faceRank[f] = r;
        a.faceByRank[r] = f;
    }
    if (bad && threadIdx.x == 0)
        atomicAdd(a.overflow, 1u << 20);
}

void launch_face_keys(const FaceOrderArgs &a, cudaStream_t s)
{
    if (a.nFaces <= 0)
        return;
    KTime kt("k_face_order", s);
    SB_COUNT(k_face_keys)<<<(a.nFaces + 255) / 256, 256, 0, s>>>(a);
}

constexpr int kFaceCtxSmemBytes = 226 * 1024; // of the 227 KB a block may take, leaving room for static arrays
static_assert(kCtxSortMax * (sizeof(unsigned long long) + sizeof(int)) <= kFaceCtxSmemBytes, "sort fits");

static int face_ctx_smem_bytes()
{
    static std::once_flag once;
    static cudaError_t attrErr = cudaSuccess;
    std::call_once(once, [] {
        attrErr = cudaFuncSetAttribute(k_face_ctx, cudaFuncAttributeMaxDynamicSharedMemorySize, kFaceCtxSmemBytes);
    });
    return attrErr == cudaSuccess ? kFaceCtxSmemBytes : 0;
}

bool face_ctx_block_sort(int FA, int FB)
{
    return std::max(FA, FB) <= kCtxSortMax && face_ctx_smem_bytes() > 0;
}

void launch_face_ctx(const FaceOrderArgs &a, cudaStream_t s)
{
    if (a.nFaces <= 0)
        return;
    const int bytes = face_ctx_smem_bytes();
    KTime kt("k_face_order", s);
    SB_COUNT(k_face_ctx)<<<2, kOrderThreads, bytes, s>>>(a, bytes / 4);
}

// ---------------------------------------------------------------------------------------------------
// per-face offsets in the processing order
// ---------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kOrderThreads) k_rank_scan(RankScanArgs a)
{
    const int k = blockIdx.x;
    int *tmp = a.tmp[k];
    for (int r = threadIdx.x; r < a.n; r += blockDim.x)
        tmp[r] = a.vals[k][a.faceByRank[r]];
    __syncthreads();
    const int total = block_excl_scan(tmp, a.n);
    for (int f = threadIdx.x; f < a.n; f += blockDim.x)
        a.out[k][f] = tmp[a.faceRank[f]];
    if (threadIdx.x == 0) {
        a.out[k][a.n] = total;
        a.tot[k][0] = a.FA < a.n ? tmp[a.FA] : total;
        a.tot[k][1] = total;
    }
}

// The multi-block form for many faces: values gathered in rank order with per-block sums (blockIdx.y = the
// array), the block sums scanned by one block, then each block scans its chunk from its offset, and the
// results are scattered back to face order.
constexpr int kRankScanBlockMax = 16384; // faces up to which one block per array scans
constexpr int kRankChunk = 1024;         // ranks per block in the multi-block form

__global__ void __launch_bounds__(kRankChunk) k_rank_gather(RankScanArgs a, int nb)
{
    const int k = blockIdx.y, r = blockIdx.x * kRankChunk + threadIdx.x;
    const int v = r < a.n ? a.vals[k][a.faceByRank[r]] : 0;
    if (r < a.n)
        a.tmp[k][r] = v;
    int s = v;
    for (int o = 16; o > 0; o >>= 1)
        s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
    __shared__ int ws[32];
    if ((threadIdx.x & 31) == 0)
        ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < kRankChunk / 32; ++w)
            t += ws[w];
        a.part[k * nb + blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(kOrderThreads) k_rank_parts(RankScanArgs a, int nb)
{
    for (int k = 0; k < a.count; ++k) {
        const int total = block_excl_scan(a.part + k * nb, nb);
        if (threadIdx.x == 0)
            a.tot[k][1] = total;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kRankChunk) k_rank_chunk_scan(RankScanArgs a, int nb)
{
    const int k = blockIdx.y, r = blockIdx.x * kRankChunk + threadIdx.x, lane = threadIdx.x & 31,
              w = threadIdx.x >> 5;
    const int v = r < a.n ? a.tmp[k][r] : 0;
    int incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o)
            incl += t;
    }
    __shared__ int ws[32];
    if (lane == 31)
        ws[w] = incl;
    __syncthreads();
    if (w == 0) {
        const int x = ws[lane];
        int y = x;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xFFFFFFFFu, y, o);
            if (lane >= o)
                y += t;
        }
        ws[lane] = y - x;
    }
    __syncthreads();
    const int excl = a.part[k * nb + blockIdx.x] + ws[w] + incl - v;
    if (r < a.n)
        a.tmp[k][r] = excl;
    if (r == a.FA && a.FA < a.n)
        a.tot[k][0] = excl;
}

__global__ void k_rank_scatter(RankScanArgs a)
{
    const int k = blockIdx.y, f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f < a.n)
        a.out[k][f] = a.tmp[k][a.faceRank[f]];
    if (f == 0) {
        a.out[k][a.n] = a.tot[k][1];
        if (a.FA >= a.n)
            a.tot[k][0] = a.tot[k][1];
    }
}

void launch_rank_scan(const RankScanArgs &a, cudaStream_t s)
{
    if (a.n <= 0 || a.count <= 0)
        return;
    KTime kt("k_rank_scan", s);
    const int nb = (a.n + kRankChunk - 1) / kRankChunk;
    if (a.n <= kRankScanBlockMax || !a.part || nb > 1024) {
        SB_COUNT(k_rank_scan)<<<a.count, kOrderThreads, 0, s>>>(a);
        return;
    }
    const dim3 g(nb, a.count);
    SB_COUNT(k_rank_gather)<<<g, kRankChunk, 0, s>>>(a, nb);
    SB_COUNT(k_rank_parts)<<<1, kOrderThreads, 0, s>>>(a, nb);
    SB_COUNT(k_rank_chunk_scan)<<<g, kRankChunk, 0, s>>>(a, nb);
    SB_COUNT(k_rank_scatter)<<<dim3((a.n + 255) / 256, a.count), 256, 0, s>>>(a);
}

// ---------------------------------------------------------------------------------------------------
// loops (buildPolygonsFromEdges, src/solidboolean.cpp:124-165) and the seeds of the face groups (:167-200)
// ---------------------------------------------------------------------------------------------------

// diagnostic: device time at phase boundaries of the one-block kernels (thread 0, after a barrier)
__device__ __forceinline__ void phase_stamp(unsigned long long *stamps, int k)
{
    if (stamps && threadIdx.x == 0) {
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        stamps[k] = t;
    }
}

constexpr int kRulerStride = 8;   // every 8th appended vertex id on a loop is a ruler
constexpr int kOrphanProbe = 64;  // a vertex that meets no ruler within this many steps becomes one

// Bump allocation of one block's work arrays: from dynamic shared memory while it lasts, else from the
// global scratch (which is sized for every array, so its offsets do not depend on what fitted).
struct Bump {
    int *sm;
    long long smLeft;
    int *gl;
    __device__ int *take(long long n)
    {
        n = (n + 3) & ~3ll; // 16-byte alignment for int2 / int4 views
        int *p;
        if (n <= smLeft) {
            p = sm;
            sm += n;
            smLeft -= n;
        } else {
            p = gl;
        }
        gl += n;
        return p;
    }
    // where take(n) would place n ints, without taking them (a temporary that later takes overwrite)
    __device__ int *peek(long long n) const { return ((n + 3) & ~3ll) <= smLeft ? sm : gl; }
};

size_t loop_order_scratch_ints(int slotDomain, int nNew)
{
    const long long N = std::max(nNew, 1), W = 2 * N + 2;
    auto r4 = [](long long n) { return (n + 3) & ~3ll; };
    // phase 1: flag; phase 3 on: adjacency, iteration positions, ruler ids, ruler vertices, 15 arrays per walk,
    // the loop flag, 4 per loop
    return (size_t)(r4(std::max<long long>(slotDomain, N) + 1) + r4(2 * N) + 3 * r4(N) + 15 * r4(W) + r4(N + 1) +
                    4 * r4(N + 1) + 64);
}

__device__ __forceinline__ int other_nb(int2 nb, int prev) { return nb.x == prev ? nb.y : nb.x; }

// One block. Loop vertices are the appended vertices on the first mesh's cut edges; every one has exactly two
// neighbours (else combine fails and nothing here runs). In the loop map a vertex is inserted as a key at its
// first occurrence in the edge sequence; the map's iteration order makes the loop list: each loop starts at
// its vertex met first in that order and goes on to the neighbour its set iterates first, which for a set of
// two is the one inserted second. Positions along the loops come from ruler walks: rulers (every 8th vertex
// id, and one vertex of each loop that has none) walk both ways to the next ruler in shared memory, then
// pointer jumping over the walks finds each loop's first vertex and ranks the walks from it.
__global__ void __launch_bounds__(kOrderThreads) k_loop_order(LoopOrderArgs a)
{
    extern __shared__ __align__(16) int dsm[];
    const int T = blockDim.x, tid = threadIdx.x;
    if (*a.loopBad != 0 || a.nNew <= 0) {
        if (tid == 0)
            a.info[0] = a.info[1] = 0;
        return;
    }
    const int nNew = a.nNew;
    __shared__ int bad;
    phase_stamp(a.stamps, 0);
    // 1. insertion sequence of the map's keys
    int *flag;
    {
        Bump b1{dsm, a.smemInts, a.scratch};
        flag = b1.take(max(a.slotDomain, nNew) + 1);
    }
    for (int i = tid; i < a.slotDomain; i += T)
        flag[i] = 0;
    __syncthreads();
    for (int x = tid; x < nNew; x += T)
        if (a.degree[x] > 0 && a.firstOcc[x] < a.slotDomain)
            flag[a.firstOcc[x]] = 1;
    __syncthreads();
    const int nLV = block_excl_scan(flag, a.slotDomain);
    for (int x = tid; x < nNew; x += T)
        if (a.degree[x] > 0 && a.firstOcc[x] < a.slotDomain) {
            const int r = flag[a.firstOcc[x]];
            a.insRank[x] = r;
            a.insKeys[r] = a.newBase + (uint32_t)x;
        }
    __syncthreads();
    phase_stamp(a.stamps, 1);
    // 2. iteration order (checked to be a permutation before anything is indexed by it)
    hash_order_block(a.insKeys, nLV, a.hashOut, a.hs, dsm, (int)a.smemInts);
    int *chk = a.scratch; // the phase-1 flag's global twin is free now
    if (tid == 0)
        bad = 0;
    for (int i = tid; i < nLV; i += T)
        chk[i] = 0;
    __syncthreads();
    for (int i = tid; i < nLV; i += T) {
        const int p = a.hashOut[i];
        if (p < 0 || p >= nLV || atomicAdd(&chk[p], 1) != 0)
            bad = 1;
    }
    __syncthreads();
    if (bad) {
        if (tid == 0) {
            a.info[0] = a.info[1] = 0;
            atomicAdd(a.loopErr, 1u);
        }
        return;
    }
    phase_stamp(a.stamps, 2);
    // 3. work arrays of the walks
    Bump bm{dsm, a.smemInts, a.scratch};
    int2 *NB = reinterpret_cast<int2 *>(bm.take(2ll * nNew));
    int *IT = bm.take(nNew), *RI = bm.take(nNew), *RV = bm.take(nNew);
    for (int x = tid; x < nNew; x += T) {
        const bool lv = a.degree[x] == 2;
        NB[x] = lv ? make_int2(a.nbr[2 * x], a.nbr[2 * x + 1]) : make_int2(-1, -1);
        IT[x] = lv ? a.hashOut[a.insRank[x]] : INT_MAX;
        RI[x] = (lv && x % kRulerStride == 0) ? 1 : 0;
    }
    __syncthreads();
    // rulers: the regular ones, plus the smallest vertex id of a loop that holds none, plus any vertex that
    // meets no ruler within the probe length
    for (int x = tid; x < nNew; x += T) {
        if (NB[x].x < 0 || RI[x])
            continue;
        int prev = x, cur = NB[x].x, mnId = x, steps = 0;
        bool hit = false;
        while (cur != x && steps < kOrphanProbe) {
            if (RI[cur] == 1) {
                hit = true;
                break;
            }
            mnId = min(mnId, cur);
            const int nx = other_nb(NB[cur], prev);
            prev = cur;
            cur = nx;
            ++steps;
        }
        if (!hit && (cur != x || mnId == x))
            RI[x] = 2; // (the probes test RI == 1 only, so this write does not disturb them)
    }
    __syncthreads();
    // ruler ids: RI[x] for rulers, -1 else; RV[id] = its vertex. The scan runs in a temporary that the walk
    // arrays take over afterwards.
    int *scanTmp = bm.peek(nNew);
    for (int x = tid; x < nNew; x += T)
        scanTmp[x] = RI[x] ? 1 : 0;
    __syncthreads();
    const int nR = block_excl_scan(scanTmp, nNew);
    for (int x = tid; x < nNew; x += T) {
        if (RI[x]) {
            RI[x] = scanTmp[x];
            RV[scanTmp[x]] = x;
        } else {
            RI[x] = -1;
        }
    }
    __syncthreads();
    const int nW = 2 * nR;
    int *wSucc = bm.take(nW), *wLen = bm.take(nW), *wMin = bm.take(nW), *wArg = bm.take(nW);
    int *cmA = bm.take(nW), *cmB = bm.take(nW), *caA = bm.take(nW), *caB = bm.take(nW);
    int *sA = bm.take(nW), *sB = bm.take(nW), *dA = bm.take(nW), *dB = bm.take(nW);
    int *wLoop = bm.take(nW), *wP = bm.take(nW), *wReach = bm.take(nW);
    int *lflag = bm.take(nLV + 1);
    phase_stamp(a.stamps, 3);
    // 4. the walks: walk w = 2 r + s leaves ruler RV[r] through its neighbour s and stops at the next ruler;
    // vertex x passed from its neighbour e records (w, offset) in vis[2 x + e]
    for (int w = tid; w < nW; w += T) {
        const int r0 = RV[w >> 1];
        int prev = r0, cur = (w & 1) ? NB[r0].y : NB[r0].x, off = 1, mn = IT[r0], arg = r0;
        for (int steps = 0; steps <= nLV && RI[cur] < 0; ++steps) {
            const int e = NB[cur].x == prev ? 0 : 1;
            a.vis[2 * cur + e] = make_int2(w, off);
            if (IT[cur] < mn) {
                mn = IT[cur];
                arg = cur;
            }
            const int nx = e == 0 ? NB[cur].y : NB[cur].x;
            prev = cur;
            cur = nx;
            ++off;
        }
        const int j = NB[cur].x == prev ? 0 : 1;
        wSucc[w] = RI[cur] >= 0 ? 2 * RI[cur] + (1 - j) : w;
        wLen[w] = off;
        wMin[w] = mn;
        wArg[w] = arg;
    }
    __syncthreads();
    int rounds = 1;
    while ((1 << rounds) < nW + 1)
        ++rounds;
    ++rounds;
    phase_stamp(a.stamps, 4);
    // 5. each loop's first vertex in iteration order: pointer jumping (min) over the walks of one orientation
    for (int w = tid; w < nW; w += T) {
        sA[w] = wSucc[w];
        cmA[w] = wMin[w];
        caA[w] = wArg[w];
    }
    __syncthreads();
    for (int r = 0; r < rounds; ++r) {
        for (int w = tid; w < nW; w += T) {
            const int sc = sA[w];
            const bool take = cmA[sc] < cmA[w];
            cmB[w] = take ? cmA[sc] : cmA[w];
            caB[w] = take ? caA[sc] : caA[w];
            sB[w] = sA[sc];
        }
        __syncthreads();
        int *t = sA;
        sA = sB;
        sB = t;
        t = cmA;
        cmA = cmB;
        cmB = t;
        t = caA;
        caA = caB;
        caB = t;
    }
    // loops in iteration order of their first vertices
    for (int i = tid; i <= nLV; i += T)
        lflag[i] = 0;
    __syncthreads();
    for (int w = tid; w < nW; w += T)
        if (cmA[w] >= 0 && cmA[w] < nLV)
            lflag[cmA[w]] = 1;
    __syncthreads();
    const int nLoops = block_excl_scan(lflag, nLV);
    int *lW0 = bm.take(nLoops + 1), *lO0 = bm.take(nLoops + 1), *lLen = bm.take(nLoops + 1);
    int *lOff = bm.take(nLoops + 1);
    for (int w = tid; w < nW; w += T) {
        const int loop = lflag[cmA[w]];
        wLoop[w] = loop;
        // the walk holding the loop's first vertex s0 in the direction the loop takes (towards the neighbour
        // inserted second), and s0's offset in it
        const int s0 = caA[w];
        const int ks = a.nbrSlot[2 * s0] > a.nbrSlot[2 * s0 + 1] ? 0 : 1;
        const int toward = ks == 0 ? a.nbr[2 * s0] : a.nbr[2 * s0 + 1];
        int W0, o0;
        if (RI[s0] >= 0) {
            W0 = 2 * RI[s0] + (NB[s0].x == toward ? 0 : 1);
            o0 = 0;
        } else {
            const int e = NB[s0].x == toward ? 1 : 0; // entered from the other neighbour
            const int2 rec = a.vis[2 * s0 + e];
            W0 = rec.x;
            o0 = rec.y;
        }
        if (W0 < 0 || W0 >= nW) { // cannot happen for loops of two-neighbour vertices; keep indices in range
            W0 = w;
            o0 = 0;
            atomicAdd(a.loopErr, 1u);
        }
        lW0[loop] = W0; // every walk of the loop writes the same values
        lO0[loop] = o0;
    }
    __syncthreads();
    phase_stamp(a.stamps, 5);
    // 6. rank the walks from the loop's first walk along its direction: cut the cycle before it, suffix sums
    for (int w = tid; w < nW; w += T) {
        const int sc = wSucc[w];
        const bool tail = sc == lW0[wLoop[w]];
        sA[w] = tail ? -1 : sc;
        dA[w] = wLen[w];
    }
    __syncthreads();
    for (int r = 0; r < rounds; ++r) {
        for (int w = tid; w < nW; w += T) {
            const int sc = sA[w];
            dB[w] = sc >= 0 ? dA[w] + dA[sc] : dA[w];
            sB[w] = sc >= 0 ? sA[sc] : -1;
        }
        __syncthreads();
        int *t = sA;
        sA = sB;
        sB = t;
        t = dA;
        dA = dB;
        dB = t;
    }
    for (int w = tid; w < nW; w += T)
        wReach[w] = sA[w] == -1 ? 1 : 0;
    __syncthreads();
    for (int w = tid; w < nW; w += T) {
        const int loop = wLoop[w];
        const int L = dA[lW0[loop]];
        wP[w] = L - dA[w]; // offset of the walk's first vertex after the first walk's first vertex
        if (w == lW0[loop])
            lLen[loop] = L;
    }
    __syncthreads();
    for (int l = tid; l < nLoops; l += T)
        lOff[l] = lLen[l];
    __syncthreads();
    block_excl_scan(lOff, nLoops);
    phase_stamp(a.stamps, 6);
    for (int i = tid; i < 2 * 2 * nLV; i += T)
        a.seedTri[i] = -1;
    for (int i = tid; i < nLV; i += T)
        a.entryLoop[i] = -1;
    __syncthreads();
    // 7. every loop vertex's place: loop position p of loop l holds edge (l_p, l_p+1); entries 2 (off_l + p)
    // and 2 (off_l + p) + 1 are its two half-edges (k_seed_entries looks their owners up, grid-wide)
    for (int x = tid; x < nNew; x += T) {
        int w = -1, o = 0, next = -1;
        if (NB[x].x >= 0) {
            if (RI[x] >= 0) {
                for (int s2 = 0; s2 < 2; ++s2)
                    if (wReach[2 * RI[x] + s2]) {
                        w = 2 * RI[x] + s2;
                        next = s2 ? NB[x].y : NB[x].x;
                    }
            } else {
                for (int e = 0; e < 2; ++e) {
                    const int2 rec = a.vis[2 * x + e];
                    if (rec.x >= 0 && rec.x < nW && wReach[rec.x]) {
                        w = rec.x;
                        o = rec.y;
                        next = e == 0 ? NB[x].y : NB[x].x;
                    }
                }
            }
        }
        int base = -1;
        if (w >= 0) {
            const int loop = wLoop[w], L = lLen[loop];
            if (L > 0) {
                int p = wP[w] + o - lO0[loop];
                p = ((p % L) + L) % L;
                base = lOff[loop] + p;
                if (base < 0 || base >= nLV)
                    base = -1;
                else
                    a.entryLoop[base] = loop;
            }
        }
        a.entryBase[x] = base;
        a.entryNext[x] = next;
    }
    if (tid == 0) {
        a.info[0] = nLV;
        a.info[1] = nLoops;
    }
    phase_stamp(a.stamps, 7);
}

// The seed entries' triangles (the owners of each loop edge's two half-edges in each mesh), and the first
// entry of every triangle. Grid-wide: the hash-table probes are latency-bound.
__global__ void k_seed_entries(LoopOrderArgs a)
{
    const int nLV = a.info[0], nLoops = a.info[1], nE = 2 * nLV;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x < 4 * nLoops) {
        a.group0[x] = INT_MAX;
        a.gQuery[x] = -1;
    }
    if (x >= a.nNew)
        return;
    const int base = a.entryBase[x];
    if (base < 0 || base >= nLV)
        return;
    const uint32_t u = a.newBase + (uint32_t)x, v = a.newBase + (uint32_t)a.entryNext[x];
    for (int m = 0; m < 2; ++m) {
        const uint64_t *hk = m ? a.heKeysB : a.heKeysA;
        const int *hv = m ? a.heValsB : a.heValsA;
        const int t0 = u64map_find(hk, hv, a.heMask, he_key(u, v));
        const int t1 = u64map_find(hk, hv, a.heMask, he_key(v, u));
        a.seedTri[m * nE + 2 * base] = t0;
        a.seedTri[m * nE + 2 * base + 1] = t1;
        if (t0 >= 0 && t0 < a.nTri)
            atomicMin(&a.firstQ[t0], 2 * base);
        if (t1 >= 0 && t1 < a.nTri)
            atomicMin(&a.firstQ[t1], 2 * base + 1);
    }
}

// each group's first triangle: its first entry whose triangle no earlier entry claimed
__global__ void k_seed_groups(LoopOrderArgs a)
{
    const int nLV = a.info[0], nLoops = a.info[1], nE = 2 * nLV;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 2 * nE)
        return;
    const int t = a.seedTri[i], q = i % nE, m = i / nE;
    if (t < 0 || t >= a.nTri || a.firstQ[t] != q)
        return;
    const int l = a.entryLoop[q >> 1];
    if (l >= 0 && l < nLoops)
        atomicMin(&a.group0[m * 2 * nLoops + 2 * l + (q & 1)], q);
}

// The side queries: every non-empty group's first triangle, and every region without seeds (one of the
// reference's remaining groups, src/solidboolean.cpp:231-238) by its smallest uncut triangle. Also counts the
// regions per mesh.
__global__ void k_side_queries(AsmArgs g, LoopOrderArgs a)
{
    const int nLV = a.info[0], nLoops = a.info[1], nE = 2 * nLV;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 4 * nLoops) {
        const int q = a.group0[i];
        if (q != INT_MAX) {
            const int m = i / (2 * nLoops);
            const unsigned int k = atomicAdd(a.qCount, 1u);
            a.qTri[k] = a.seedTri[m * nE + q];
            a.gQuery[i] = (int)k;
        }
    }
    if (i >= g.nTri || g.parent[i] != i)
        return;
    g.repOfRoot[i] = -1;
    if (g.seedMin[i] != INT_MAX) {
        atomicAdd(g.counters + kCntRegionsA + g.triMesh[i], 1u);
        return;
    }
    if (g.remMin[i] != INT_MAX) {
        const unsigned int k = atomicAdd(a.qCount, 1u);
        a.qTri[k] = g.remMin[i];
        g.repOfRoot[i] = (int)k;
        atomicAdd(g.counters + kCntRegionsA + g.triMesh[i], 1u);
    }
}

constexpr int kOrderSmemBytes = 226 * 1024; // of the 227 KB a block may take, leaving room for static arrays

void launch_loop_order(LoopOrderArgs a, cudaStream_t s)
{
    static std::once_flag once;
    static cudaError_t attrErr = cudaSuccess;
    std::call_once(once, [] {
        attrErr = cudaFuncSetAttribute(k_loop_order, cudaFuncAttributeMaxDynamicSharedMemorySize, kOrderSmemBytes);
    });
    a.smemInts = attrErr == cudaSuccess ? kOrderSmemBytes / 4 : 0;
    KTime kt("k_loop_order", s);
    SB_COUNT(k_loop_order)<<<1, kOrderThreads, attrErr == cudaSuccess ? kOrderSmemBytes : 0, s>>>(a);
}

void launch_seed_entries(const LoopOrderArgs &a, cudaStream_t s)
{
    const int n = std::max(a.nNew, 1);
    KTime kt("k_seed_entries", s);
    SB_COUNT(k_seed_entries)<<<(n + 255) / 256, 256, 0, s>>>(a);
    SB_COUNT(k_seed_groups)<<<(4 * n + 255) / 256, 256, 0, s>>>(a);
}

void launch_side_queries(const AsmArgs &g, const LoopOrderArgs &a, cudaStream_t s)
{
    const int n = std::max(g.nTri, 4 * std::max(a.nNew, 1));
    KTime kt("k_side_queries", s);
    SB_COUNT(k_side_queries)<<<(n + 255) / 256, 256, 0, s>>>(g, a);
}

// ---------------------------------------------------------------------------------------------------
// sides of regions, the exact flood of mixed regions, labels
// ---------------------------------------------------------------------------------------------------
__device__ __forceinline__ int query_side(const int *insideCount, int k)
{
    return ((float)insideCount[k] / 3.0f > 0.5f) ? 1 : 0; // (float)inside / total > 0.5
}

// live entry (i = m * nE + q): the first entry of its triangle
__device__ __forceinline__ bool entry_live(const FloodArgs &f, int i, int nE, int &t, int &group)
{
    t = f.seedTri[i];
    const int q = i % nE;
    if (t < 0 || t >= f.nTri || f.firstQ[t] != q)
        return false;
    const int l = f.entryLoop[q >> 1];
    if (l < 0 || l >= f.info[1])
        return false;
    group = 2 * l + (q & 1);
    return true;
}

__global__ void k_region_sides(FloodArgs f)
{
    const int nE = 2 * f.info[0], nLoops = f.info[1];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * nE; i += gridDim.x * blockDim.x) {
        int t, grp;
        if (!entry_live(f, i, nE, t, grp))
            continue;
        const int m = i / nE;
        const int k = f.gQuery[m * 2 * nLoops + grp];
        if (k < 0)
            continue;
        const int side = query_side(f.insideCount, k);
        const int r = f.root[t];
        atomicMin(&f.rsMin[r], side);
        atomicMax(&f.rsMax[r], side);
    }
}

__device__ __forceinline__ bool mixed_region(const FloodArgs &f, int r) { return f.rsMin[r] == 0 && f.rsMax[r] == 1; }

// Level 0 of the flood, grid-wide: flag i (mesh i & 1, entry i >> 1) marks a live entry of a region whose groups
// were decided differently; anyMixed records whether there is one (usually not: then the flood does nothing).
__global__ void k_flood_seeds(FloodArgs f)
{
    const int nE = 2 * f.info[0], nI = 2 * nE;
    bool any = false;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nI; i += gridDim.x * blockDim.x) {
        const int m = i & 1, q = i >> 1;
        int t, grp;
        const int on = (entry_live(f, m * nE + q, nE, t, grp) && mixed_region(f, f.root[t])) ? 1 : 0;
        f.flag[i] = on;
        any |= on != 0;
    }
    if (__any_sync(0xFFFFFFFFu, any) && (threadIdx.x & 31) == 0)
        atomicOr(f.anyMixed, 1);
}

// One block: the reference's first-in-first-out flood (src/solidboolean.cpp:205-233) restricted to the
// regions whose groups were decided differently, level by level. A level's queue is its triangles in pop
// order; a triangle first reached at the next level is pushed by the earliest (parent, edge) in that order,
// so it takes the group of the smallest key 3 * parent position + edge, and the next queue lists the newly
// reached triangles by that key. The seeds are the live entries of those regions in entry order.
__global__ void __launch_bounds__(kOrderThreads) k_flood(AsmArgs g, FloodArgs f)
{
    const int T = blockDim.x, tid = threadIdx.x;
    const int nE = 2 * f.info[0];
    if (nE == 0 || *f.anyMixed == 0)
        return; // every region's groups agree: nothing to flood
    __shared__ int nFront;
    // level 0: live entries of mixed regions (flagged by k_flood_seeds), ordered by entry (both meshes
    // interleaved: they never meet)
    const int nI = 2 * nE;
    const int n0 = block_excl_scan(f.flag, nI);
    for (int i = tid; i < nI; i += T) {
        const int m = i & 1, q = i >> 1;
        int t, grp;
        if (entry_live(f, m * nE + q, nE, t, grp) && mixed_region(f, f.root[t])) {
            f.front0[f.flag[i]] = t;
            f.bfsGroup[t] = grp;
        }
    }
    if (tid == 0)
        nFront = n0;
    __syncthreads();
    int *F = f.front0, *G = f.front1;
    for (int level = 0; level < f.nTri + 1; ++level) {
        const int n = nFront;
        if (n == 0)
            break;
        for (int k = tid; k < 3 * n; k += T) {
            const int t = F[k / 3];
            const int u = arr_twin(g, t, k % 3);
            f.tgt[k] = -1;
            if (u >= 0 && f.bfsGroup[u] < 0) {
                f.tgt[k] = u;
                atomicMin(&f.best[u], k);
            }
        }
        __syncthreads();
        for (int k = tid; k < 3 * n; k += T) {
            const int u = f.tgt[k];
            f.flag[k] = (u >= 0 && f.best[u] == k) ? 1 : 0;
        }
        __syncthreads();
        const int nn = block_excl_scan(f.flag, 3 * n);
        for (int k = tid; k < 3 * n; k += T) {
            const int u = f.tgt[k];
            if (u >= 0 && f.best[u] == k) {
                G[f.flag[k]] = u;
                f.bfsGroup[u] = f.bfsGroup[F[k / 3]];
            }
        }
        if (tid == 0)
            nFront = nn;
        __syncthreads();
        int *t = F;
        F = G;
        G = t;
        if (level == f.nTri && tid == 0)
            atomicAdd(f.errors, 1u);
    }
}

__global__ void k_labels_ref(AsmArgs g, FloodArgs f)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= f.nTri)
        return;
    const int r = f.root[t];
    int8_t lab = -1;
    if (f.seedMin[r] == INT_MAX) {
        const int k = f.regionQuery[r];
        lab = k >= 0 ? (int8_t)query_side(f.insideCount, k) : (int8_t)-1;
    } else if (f.rsMin[r] == f.rsMax[r]) {
        lab = (int8_t)f.rsMin[r];
    } else if (mixed_region(f, r)) {
        const int grp = f.bfsGroup[t];
        if (grp >= 0) {
            const int k = f.gQuery[g.triMesh[t] * 2 * f.info[1] + grp];
            lab = k >= 0 ? (int8_t)query_side(f.insideCount, k) : (int8_t)-1;
        }
    }
    g.label[t] = lab;
}

void launch_flood_labels(const AsmArgs &g, const FloodArgs &f, cudaStream_t s)
{
    if (f.nTri <= 0)
        return;
    KTime kt("k_flood", s);
    SB_COUNT(k_region_sides)<<<152, 256, 0, s>>>(f);
    SB_COUNT(k_flood_seeds)<<<152, 256, 0, s>>>(f);
    SB_COUNT(k_flood)<<<1, kOrderThreads, 0, s>>>(g, f);
    SB_COUNT(k_labels_ref)<<<(f.nTri + 255) / 256, 256, 0, s>>>(g, f);
}

} // namespace sbg
