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
    return 6 * N + 1 + 3 * (size_t)hash_bucket_count((uint32_t)N) + 8;
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
    h.firstOld = h.runSize + 2 * N + 1;
    h.createNew = h.firstOld + B;
    h.head = h.createNew + B;
    return h;
}

// keys[i]: the i-th inserted key (distinct); out[i]: its position in the container's iteration order
__device__ void hash_order_block(const uint32_t *keys, int n, int *out, HashScratch w)
{
    const int T = blockDim.x, tid = threadIdx.x;
    if (n <= 0)
        return;
    int *pos = w.posA, *npos = w.posB;
    int Mprev = 0;
    for (int stage = 0; stage < 64; ++stage) {
        const uint32_t B = hash_bucket_count((uint32_t)Mprev + 1);
        const int M = (uint32_t)n < B ? n : (int)B;
        for (uint32_t b = tid; b < B; b += T) {
            w.firstOld[b] = INT_MAX;
            w.createNew[b] = INT_MAX;
            w.head[b] = -1;
        }
        for (int i = tid; i < M + Mprev; i += T)
            w.runSize[i] = 0;
        __syncthreads();
        for (int i = tid; i < M; i += T) {
            const uint32_t b = keys[i] % B;
            if (i < Mprev)
                atomicMin(&w.firstOld[b], pos[i]);
            else
                atomicMin(&w.createNew[b], i);
            w.nxt[i] = atomicExch(&w.head[b], i);
        }
        __syncthreads();
        // runs: opened by this stage's inserts [0, M - Mprev), latest first; rebuilt [M, M + Mprev)
        for (int i = tid; i < M; i += T) {
            const uint32_t b = keys[i] % B;
            const int fo = w.firstOld[b];
            const int slot = fo != INT_MAX ? M + (Mprev - 1 - fo) : (M - 1 - w.createNew[b]);
            w.slotOf[i] = slot;
            atomicAdd(&w.runSize[slot], 1);
        }
        __syncthreads();
        block_excl_scan(w.runSize, M + Mprev);
        for (int i = tid; i < M; i += T) {
            const uint32_t b = keys[i] % B;
            const int gi = i < Mprev ? 1 : 0;
            const int ki = gi ? (Mprev - 1 - pos[i]) : (M - 1 - i);
            int within = 0;
            for (int j = w.head[b]; j >= 0; j = w.nxt[j]) {
                if (j == i)
                    continue;
                const int gj = j < Mprev ? 1 : 0;
                const int kj = gj ? (Mprev - 1 - pos[j]) : (M - 1 - j);
                within += (gj < gi || (gj == gi && kj < ki)) ? 1 : 0;
            }
            npos[i] = w.runSize[w.slotOf[i]] + within;
        }
        __syncthreads();
        int *t = pos;
        pos = npos;
        npos = t;
        Mprev = M;
        if (M == n)
            break;
    }
    __syncthreads();
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
__global__ void __launch_bounds__(kOrderThreads) k_face_ctx(FaceOrderArgs a)
{
    const int side = blockIdx.x;
    const int off = side ? a.FA : 0, n = side ? a.FB : a.FA;
    uint32_t *keys = a.insKeys + off;
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        keys[i] = (uint32_t)a.faceTri[a.sortedVal[off + i]];
    __syncthreads();
    const HashScratch w = a.hs[side];
    // the result lands in slotOf, which the stages no longer need when it is written
    hash_order_block(keys, n, w.slotOf, w);
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

void launch_face_ctx(const FaceOrderArgs &a, cudaStream_t s)
{
    if (a.nFaces <= 0)
        return;
    KTime kt("k_face_order", s);
    SB_COUNT(k_face_ctx)<<<2, kOrderThreads, 0, s>>>(a);
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

void launch_rank_scan(const RankScanArgs &a, cudaStream_t s)
{
    if (a.n <= 0 || a.count <= 0)
        return;
    KTime kt("k_rank_scan", s);
    SB_COUNT(k_rank_scan)<<<a.count, kOrderThreads, 0, s>>>(a);
}

// ---------------------------------------------------------------------------------------------------
// loops (buildPolygonsFromEdges, src/solidboolean.cpp:124-165) and the seeds of the face groups (:167-200)
// ---------------------------------------------------------------------------------------------------
size_t loop_order_flag_ints(int slotDomain, int nNew) { return (size_t)std::max(slotDomain, nNew) + 1; }

// directed loop edge d = 2 x + k (x's k-th neighbour) -> the next directed edge along the loop, -1 if none
__device__ __forceinline__ int loop_succ(const int *nbr, const int *degree, int d)
{
    const int x = d >> 1;
    if (degree[x] != 2)
        return -1;
    const int v = nbr[d];
    if (v < 0 || degree[v] != 2)
        return -1;
    const int j = nbr[2 * v] == x ? 0 : 1;
    return 2 * v + (1 - j);
}

// One block. Loop vertices are the appended vertices on the first mesh's cut edges; every one has exactly two
// neighbours (else combine fails and nothing here runs). In the loop map a vertex is inserted as a key at its
// first occurrence in the edge sequence; the map's iteration order makes the loop list: each loop starts at
// its vertex met first in that order and goes on to the neighbour its set iterates first, which for a set of
// two is the one inserted second.
__global__ void __launch_bounds__(kOrderThreads) k_loop_order(LoopOrderArgs a)
{
    const int T = blockDim.x, tid = threadIdx.x;
    if (*a.loopBad != 0 || a.nNew <= 0) {
        if (tid == 0)
            a.info[0] = a.info[1] = 0;
        return;
    }
    const int nNew = a.nNew, nD = 2 * nNew;
    // 1. insertion sequence of the map's keys
    for (int i = tid; i < a.slotDomain; i += T)
        a.flag[i] = 0;
    __syncthreads();
    for (int x = tid; x < nNew; x += T)
        if (a.degree[x] > 0)
            a.flag[a.firstOcc[x]] = 1;
    __syncthreads();
    const int nLV = block_excl_scan(a.flag, a.slotDomain);
    for (int x = tid; x < nNew; x += T)
        if (a.degree[x] > 0) {
            const int r = a.flag[a.firstOcc[x]];
            a.insRank[x] = r;
            a.insKeys[r] = a.newBase + (uint32_t)x;
        }
    __syncthreads();
    // 2. iteration order (checked to be a permutation before anything is indexed by it)
    hash_order_block(a.insKeys, nLV, a.hashOut, a.hs);
    __shared__ int bad;
    if (tid == 0)
        bad = 0;
    for (int i = tid; i < nLV; i += T)
        a.flag[i] = 0;
    __syncthreads();
    for (int i = tid; i < nLV; i += T) {
        const int p = a.hashOut[i];
        if (p < 0 || p >= nLV || atomicAdd(&a.flag[p], 1) != 0)
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
    for (int x = tid; x < nNew; x += T)
        a.iterPos[x] = a.degree[x] > 0 ? a.hashOut[a.insRank[x]] : INT_MAX;
    __syncthreads();
    int rounds = 1;
    while ((1 << rounds) < nLV + 1)
        ++rounds;
    ++rounds;
    // 3. smallest iteration position on each loop (pointer jumping over the directed edges)
    for (int d = tid; d < nD; d += T) {
        a.succA[d] = loop_succ(a.nbr, a.degree, d);
        a.valA[d] = a.iterPos[d >> 1];
    }
    __syncthreads();
    int *sA = a.succA, *sB = a.succB, *vA = a.valA, *vB = a.valB;
    for (int r = 0; r < rounds; ++r) {
        for (int d = tid; d < nD; d += T) {
            const int s = sA[d];
            vB[d] = s >= 0 ? min(vA[d], vA[s]) : vA[d];
            sB[d] = s >= 0 ? sA[s] : -1;
        }
        __syncthreads();
        int *t = sA;
        sA = sB;
        sB = t;
        t = vA;
        vA = vB;
        vB = t;
    }
    for (int d = tid; d < nD; d += T)
        a.cyc[d] = vA[d];
    // 4. loop starts in iteration order, the start edges, and the edge that closes each loop
    for (int i = tid; i <= nLV; i += T)
        a.flag[i] = 0;
    __syncthreads();
    for (int x = tid; x < nNew; x += T)
        if (a.degree[x] == 2 && a.iterPos[x] == a.cyc[2 * x])
            a.flag[a.iterPos[x]] = 1;
    __syncthreads();
    const int nLoops = block_excl_scan(a.flag, nLV);
    // ranking: distance of every directed edge to the closing edge of its loop's start orientation
    for (int d = tid; d < nD; d += T) {
        const int s = loop_succ(a.nbr, a.degree, d);
        bool tail = false;
        if (s >= 0) {
            const int v = s >> 1;
            if (a.iterPos[v] == a.cyc[2 * v]) {
                const int ks = a.nbrSlot[2 * v] > a.nbrSlot[2 * v + 1] ? 0 : 1; // inserted later iterates first
                tail = (s & 1) == ks;
            }
        }
        sA[d] = tail ? -1 : s;
        vA[d] = (tail || s < 0) ? 0 : 1;
    }
    __syncthreads();
    for (int r = 0; r < rounds; ++r) {
        for (int d = tid; d < nD; d += T) {
            const int s = sA[d];
            vB[d] = s >= 0 ? vA[d] + vA[s] : vA[d];
            sB[d] = s >= 0 ? sA[s] : -1;
        }
        __syncthreads();
        int *t = sA;
        sA = sB;
        sB = t;
        t = vA;
        vA = vB;
        vB = t;
    }
    // loop lengths (at each start edge: distance + 1), then loop offsets
    for (int x = tid; x < nNew; x += T)
        if (a.degree[x] == 2 && a.iterPos[x] == a.cyc[2 * x]) {
            const int ks = a.nbrSlot[2 * x] > a.nbrSlot[2 * x + 1] ? 0 : 1;
            a.loopLen[a.flag[a.iterPos[x]]] = vA[2 * x + ks] + 1;
        }
    __syncthreads();
    block_excl_scan(a.loopLen, nLoops);
    // 5. seed entries: loop position p of loop l holds edge (l_p, l_p+1); its two half-edges' owners in each
    // mesh are entries 2 (off_l + p) and 2 (off_l + p) + 1
    const int nE = 2 * nLV;
    for (int d = tid; d < nD; d += T) {
        if (sA[d] != -1 || a.degree[d >> 1] != 2)
            continue;
        const int s0 = loop_succ(a.nbr, a.degree, d);
        if (s0 < 0)
            continue;
        const int loop = a.flag[a.cyc[d]];
        const int end = loop + 1 < nLoops ? a.loopLen[loop + 1] : nLV;
        const int L = end - a.loopLen[loop];
        const int p = L - 1 - vA[d];
        if (p < 0 || p >= L)
            continue;
        const int base = a.loopLen[loop] + p;
        a.entryLoop[base] = loop;
        const uint32_t u = a.newBase + (uint32_t)(d >> 1), v = a.newBase + (uint32_t)a.nbr[d];
        for (int m = 0; m < 2; ++m) {
            const uint64_t *hk = m ? a.heKeysB : a.heKeysA;
            const int *hv = m ? a.heValsB : a.heValsA;
            a.seedTri[m * nE + 2 * base] = u64map_find(hk, hv, a.heMask, he_key(u, v));
            a.seedTri[m * nE + 2 * base + 1] = u64map_find(hk, hv, a.heMask, he_key(v, u));
        }
    }
    __syncthreads();
    for (int i = tid; i < 2 * nE; i += T) {
        const int t = a.seedTri[i];
        if (t >= 0)
            atomicMin(&a.firstQ[t], i % nE);
    }
    for (int i = tid; i < 2 * 2 * nLoops; i += T) {
        a.group0[i] = INT_MAX;
        a.gQuery[i] = -1;
    }
    __syncthreads();
    // 6. each group's first triangle: its first entry whose triangle no earlier entry claimed
    for (int i = tid; i < 2 * nE; i += T) {
        const int t = a.seedTri[i], q = i % nE, m = i / nE;
        if (t >= 0 && a.firstQ[t] == q)
            atomicMin(&a.group0[m * 2 * nLoops + 2 * a.entryLoop[q >> 1] + (q & 1)], q);
    }
    __syncthreads();
    for (int i = tid; i < 2 * 2 * nLoops; i += T) {
        const int q = a.group0[i];
        if (q == INT_MAX)
            continue;
        const int m = i / (2 * nLoops);
        const unsigned int k = atomicAdd(a.qCount, 1u);
        a.qTri[k] = a.seedTri[m * nE + q];
        a.gQuery[i] = (int)k;
    }
    if (tid == 0) {
        a.info[0] = nLV;
        a.info[1] = nLoops;
    }
}

void launch_loop_order(const LoopOrderArgs &a, cudaStream_t s)
{
    KTime kt("k_loop_order", s);
    SB_COUNT(k_loop_order)<<<1, kOrderThreads, 0, s>>>(a);
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
    if (t < 0 || f.firstQ[t] != q)
        return false;
    group = 2 * f.entryLoop[q >> 1] + (q & 1);
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

// One block: the reference's first-in-first-out flood (src/solidboolean.cpp:205-233) restricted to the
// regions whose groups were decided differently, level by level. A level's queue is its triangles in pop
// order; a triangle first reached at the next level is pushed by the earliest (parent, edge) in that order,
// so it takes the group of the smallest key 3 * parent position + edge, and the next queue lists the newly
// reached triangles by that key. The seeds are the live entries of those regions in entry order.
__global__ void __launch_bounds__(kOrderThreads) k_flood(AsmArgs g, FloodArgs f)
{
    const int T = blockDim.x, tid = threadIdx.x;
    const int nE = 2 * f.info[0];
    if (nE == 0)
        return;
    __shared__ int nFront;
    // level 0: live entries of mixed regions, ordered by entry (both meshes interleaved: they never meet)
    const int nI = 2 * nE;
    for (int i = tid; i < nI; i += T) {
        const int m = i & 1, q = i >> 1;
        int t, grp;
        f.flag[i] = (entry_live(f, m * nE + q, nE, t, grp) && mixed_region(f, f.root[t])) ? 1 : 0;
    }
    __syncthreads();
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
    SB_COUNT(k_flood)<<<1, kOrderThreads, 0, s>>>(g, f);
    SB_COUNT(k_labels_ref)<<<(f.nTri + 255) / 256, 256, 0, s>>>(g, f);
}

} // namespace sbg
