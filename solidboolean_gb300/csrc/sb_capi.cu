// C ABI and host orchestration of the GB300 boolean (see include/solidboolean_gb300.h).
//
// combine() is the reference's SolidBoolean::combine (src/solidboolean.cpp:288-480) as a sequence of
// device stages on one stream: broad phase, narrow phase, per-face re-triangulation, global weld,
// arrangement, cut-loop check, union-find regions, side rays, fetch compaction. The host only reads the
// handful of counts that size the next stage (candidates, intersecting pairs, faces, per-face totals).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <unordered_map>
#include <thread>
#include <string>
#include <vector>

#include <cub/cub.cuh>
#include <thrust/iterator/counting_iterator.h>

#include "sb_assemble.cuh"
#include "sb_common.cuh"
#include "sb_faces.cuh"
#include "sb_internal.h"
#include "sb_order.cuh"
#include "sb_pairs.cuh"

namespace sbg {

static thread_local std::string g_last_error;
static std::atomic<unsigned long long> g_launches{0};

void set_last_error(const std::string &msg) { g_last_error = msg; }
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

// ---- per-kernel timing registry ----------------------------------------------------------------------
struct KRec {
    std::string name;
    cudaEvent_t a, b;
};
static std::mutex g_kt_mutex;
static std::vector<KRec> g_kt_recs;
static size_t g_kt_used = 0;
static std::atomic<bool> g_kt_on{false};
static std::string g_kt_only; // ",name,name," or empty for every kernel

bool ktime_enabled() { return g_kt_on.load(std::memory_order_relaxed); }

int ktime_begin(const char *name, cudaStream_t s)
{
    std::lock_guard<std::mutex> lk(g_kt_mutex);
    if (!g_kt_only.empty() && g_kt_only.find("," + std::string(name) + ",") == std::string::npos)
        return -1;
    if (g_kt_used == g_kt_recs.size()) {
        KRec r;
        if (cudaEventCreate(&r.a) != cudaSuccess || cudaEventCreate(&r.b) != cudaSuccess)
            return -1;
        g_kt_recs.push_back(r);
    }
    KRec &r = g_kt_recs[g_kt_used];
    r.name = name;
    cudaEventRecord(r.a, s);
    return (int)g_kt_used++;
}

void ktime_end(int id, cudaStream_t s)
{
    std::lock_guard<std::mutex> lk(g_kt_mutex);
    if (id >= 0 && (size_t)id < g_kt_used)
        cudaEventRecord(g_kt_recs[id].b, s);
}

sb_status cuda_fail(cudaError_t e, const char *expr, const char *file, int line)
{
    set_last_error(std::string(cudaGetErrorString(e)) + " in " + expr + " (" + file + ":" + std::to_string(line) +
                   ")");
    return SB_ERR_CUDA;
}

// Device blocks released by handles are kept per device for reuse (handles are created and destroyed per
// call on the host-buffer path, and cudaMalloc / cudaFree are slow and synchronising). A block goes back to
// the cache only after the device has finished all queued work, as cudaFree would have waited, so no later
// owner can overlap an earlier one's kernels. At most kCacheBytes stay cached.
namespace {
struct BlockCache {
    std::mutex mu;
    std::multimap<std::pair<int, size_t>, void *> free; // (device, bytes) -> block
    size_t cached = 0;
};
BlockCache g_blocks;
constexpr size_t kCacheBytes = 8ull << 30;
} // namespace

cudaError_t DevBuf::ensure(size_t need)
{
    if (need <= bytes && ptr)
        return cudaSuccess;
    release();
    const size_t n = std::max<size_t>(need + need / 4, 1024);
    int dev = 0;
    cudaGetDevice(&dev);
    {
        std::lock_guard<std::mutex> lk(g_blocks.mu);
        auto it = g_blocks.free.lower_bound({dev, need});
        if (it != g_blocks.free.end() && it->first.first == dev && it->first.second <= 2 * n) {
            ptr = it->second;
            bytes = it->first.second;
            g_blocks.cached -= bytes;
            g_blocks.free.erase(it);
            return cudaSuccess;
        }
    }
    cudaError_t e = cudaMalloc(&ptr, n);
    if (e != cudaSuccess) {
        ptr = nullptr;
        bytes = 0;
        return e;
    }
    bytes = n;
    return cudaSuccess;
}

void DevBuf::release()
{
    if (ptr) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceSynchronize(); // queued work may still use the block
        std::lock_guard<std::mutex> lk(g_blocks.mu);
        if (g_blocks.cached + bytes <= kCacheBytes) {
            g_blocks.free.insert({{dev, bytes}, ptr});
            g_blocks.cached += bytes;
        } else {
            cudaFree(ptr);
        }
    }
    ptr = nullptr;
    bytes = 0;
}

// The prepared arrays of a mesh (the layout prepare_begin carves), then one 256-byte slot for the
// validation flag, so that creating a mesh allocates nothing else (a temporary buffer that preparation later
// outgrows would be released, and a release waits for the device).
static size_t mesh_layout_bytes(int nv, int nt)
{
    Carve c;
    c.take<double>((size_t)nv * 3);
    c.take<uint32_t>((size_t)nt * 3);
    c.take<float4>((size_t)nv);
    c.take<double>((size_t)nt * 6);
    c.take<float>((size_t)nt * 6);
    c.take<uint32_t>((size_t)nt);
    c.take<int>((size_t)nt);
    c.take<int2>((size_t)(nt > 1 ? nt - 1 : 1));
    c.take<int>((size_t)(2 * nt));
    c.take<float>((size_t)(nt > 1 ? nt - 1 : 1) * 8);
    c.take<double>((size_t)(nt > 1 ? nt - 1 : 1) * 6);
    c.take<int>((size_t)(nt > 1 ? nt - 1 : 1));
    c.take<int>((size_t)nt);
    c.take<int>((size_t)nt * 3);
    c.take<int>(1);
    return c.off;
}
static size_t mesh_bytes(int nv, int nt) { return mesh_layout_bytes(nv, nt) + 256; }

static uint32_t pow2_at_least(size_t n)
{
    uint32_t p = 1024;
    while (p < n)
        p <<= 1;
    return p;
}

static inline int blocks(size_t n, int bs) { return (int)((n + bs - 1) / bs); }

// ---- small helper kernels ---------------------------------------------------------------------------
__global__ void k_validate_tris(int nt, int nv, const uint32_t *t, unsigned int *bad)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * nt)
        return;
    if (t[i] >= (uint32_t)nv)
        atomicAdd(bad, 1u);
}

__global__ void k_iota(int n, int *a)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        a[i] = i;
}

__global__ void k_fill_i32(size_t n, int *a, int v)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        a[i] = v;
}

__global__ void k_fill_u64(size_t n, uint64_t *a, uint64_t v)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        a[i] = v;
}

// Several buffers initialised by one launch (32-bit values, 64-bit values, index sequences): a small
// boolean's setup is otherwise a dozen back-to-back launches of a few microseconds each.
struct FillSeg {
    void *p;
    size_t n;
    unsigned long long v;
    int kind; // 0: 32-bit value, 1: 64-bit value, 2: a[i] = i
};
constexpr int kFillSegs = 12;
struct FillList {
    FillSeg seg[kFillSegs];
    int count;
};

__global__ void k_fill_many(FillList f)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (int k = 0; k < f.count; ++k) {
        const FillSeg sg = f.seg[k];
        for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < sg.n; i += stride) {
            if (sg.kind == 1)
                static_cast<uint64_t *>(sg.p)[i] = sg.v;
            else if (sg.kind == 2)
                static_cast<int *>(sg.p)[i] = (int)i;
            else
                static_cast<int *>(sg.p)[i] = (int)(unsigned)sg.v;
        }
    }
}

class Fills {
public:
    explicit Fills(cudaStream_t s) : s_(s) { f_.count = 0; }
    void i32(int *p, size_t n, int v) { add(p, n, (unsigned long long)(unsigned)v, 0); }
    void u64(uint64_t *p, size_t n, uint64_t v) { add(p, n, v, 1); }
    void iota(int *p, size_t n) { add(p, n, 0, 2); }
    void launch()
    {
        if (f_.count == 0)
            return;
        const size_t b = std::min<size_t>((most_ + 255) / 256, 152 * 8);
        SB_COUNT(k_fill_many)<<<(unsigned)std::max<size_t>(b, 1), 256, 0, s_>>>(f_);
        f_.count = 0;
        most_ = 0;
    }

private:
    void add(void *p, size_t n, unsigned long long v, int kind)
    {
        if (n == 0)
            return;
        if (f_.count == kFillSegs)
            launch();
        f_.seg[f_.count++] = FillSeg{p, n, v, kind};
        most_ = std::max(most_, n);
    }
    cudaStream_t s_;
    FillList f_;
    size_t most_ = 0;
};

// intersecting pair j: keys ordering its pairs inside the first mesh's face (by the second triangle's order
// key) and inside the second mesh's face (by the first triangle's order key)
// K: the number of intersecting pairs, or a bound on it with the count itself in dK (device memory)
__global__ void k_pair_keys(int K, const unsigned int *dK, const int *__restrict__ sel,
                            const uint64_t *__restrict__ cand, int nB, const int *__restrict__ rankA,
                            const int *__restrict__ rankB, const double *__restrict__ seg,
                            const uint32_t *__restrict__ perm, uint64_t *keyA, uint64_t *keyB, int *val,
                            double *segK, uint32_t *pairAB, uint32_t *pairPerm)
{
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= (dK ? (int)*dK : K))
        return;
    int idx = sel[j];
    uint64_t key = cand[idx];
    uint32_t a = (uint32_t)(key / (uint64_t)nB);
    uint32_t b = (uint32_t)(key - (uint64_t)a * (uint64_t)nB);
    uint32_t oa = rankA ? (uint32_t)rankA[a] : a;
    uint32_t ob = rankB ? (uint32_t)rankB[b] : b;
    keyA[j] = ((uint64_t)a << 32) | ob;
    keyB[j] = ((uint64_t)b << 32) | oa;
    val[j] = j;
    for (int k = 0; k < 6; ++k)
        segK[6 * (size_t)j + k] = seg[6 * (size_t)idx + k];
    pairAB[2 * (size_t)j] = a;
    pairAB[2 * (size_t)j + 1] = b;
    pairPerm[j] = perm[idx];
}

// Each cut face's pairs in the reference's processing order. Its dual traversal reaches a first-mesh face's
// pairs in the second tree's leaf order and a second-mesh face's in the first tree's, so a face's pairs sort by
// the other triangle's leaf position. The faces are grouped before the leaf orders are ready (pairs listed by
// the other triangle's index); then one thread per face sorts its list in place, in registers for up to
// kPairSortLocal pairs (the usual case: two or three), else in global memory.
constexpr int kPairSortLocal = 48;
__global__ void k_face_pair_order(int nFaces, int FA, const int *__restrict__ faceBegin, int *pairIdx,
                                  const uint32_t *__restrict__ pairAB, const int *__restrict__ rankA,
                                  const int *__restrict__ rankB)
{
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nFaces)
        return;
    const int side = f >= FA ? 1 : 0;
    const int *rank = side ? rankA : rankB; // the other mesh's leaf positions
    const int b0 = faceBegin[f], n = faceBegin[f + 1] - b0;
    auto keyOf = [&](int pair) -> uint64_t {
        const uint32_t other = pairAB[2 * (size_t)pair + (side ? 0 : 1)];
        return ((uint64_t)(uint32_t)rank[other] << 32) | (uint32_t)pair;
    };
    if (n <= 1)
        return;
    if (n <= kPairSortLocal) {
        uint64_t v[kPairSortLocal];
        for (int i = 0; i < n; ++i) {
            const uint64_t x = keyOf(pairIdx[b0 + i]);
            int j = i - 1;
            while (j >= 0 && v[j] > x) {
                v[j + 1] = v[j];
                --j;
            }
            v[j + 1] = x;
        }
        for (int i = 0; i < n; ++i)
            pairIdx[b0 + i] = (int)(uint32_t)v[i];
        return;
    }
    for (int i = 1; i < n; ++i) {
        const int pi = pairIdx[b0 + i];
        const uint64_t ki = keyOf(pi);
        int j = i - 1;
        while (j >= 0) {
            const int pj = pairIdx[b0 + j];
            if (keyOf(pj) <= ki)
                break;
            pairIdx[b0 + j + 1] = pj;
            --j;
        }
        pairIdx[b0 + j + 1] = pi;
    }
}

__global__ void k_hi32(int n, const uint64_t *__restrict__ k, int *out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        out[i] = (int)(k[i] >> 32);
}

// Groups the intersecting pairs by cut face when one side's pairs fit one block: a block radix sort of the
// compacted keys (face << orderBits | the other triangle), then the runs of equal face (unique faces, their
// pair counts and how many there are), in one launch. Block 0 takes the first mesh's faces, block 1 the
// second's; the pair indices land in pairIdx[side * K + i]. With faceOnly the sort skips the low bits: the
// pairs of each face are put in the reference's order afterwards (k_face_pair_order, by the other triangle's
// leaf position), so only the grouping counts, and the sort takes half the passes.
constexpr int kGroupThreads = 512;
constexpr int kGroupItems = 16;
constexpr int kGroupMax = kGroupThreads * kGroupItems;
using GroupSort = cub::BlockRadixSort<unsigned long long, kGroupThreads, kGroupItems, int>;
union GroupSmem {
    typename GroupSort::TempStorage sort;
    int starts[kGroupMax + 1];
};

__global__ void __launch_bounds__(kGroupThreads)
    k_face_group(int Kin, const unsigned int *dK, const uint64_t *__restrict__ keyA,
                 const uint64_t *__restrict__ keyB, const int *__restrict__ val, int orderBitsA, int orderBitsB,
                 int endBitA, int endBitB, bool faceOnly, int *pairIdx, int *uqA, int *ctA, int *uqB, int *ctB,
                 unsigned int *runCount)
{
    const int K = dK ? (int)*dK : Kin; // with dK, Kin bounds it
    if (K > kGroupMax) { // beyond one block: the host groups them device-wide once it has read the count
        if (threadIdx.x == 0)
            runCount[blockIdx.x] = 0;
        return;
    }
    extern __shared__ __align__(16) unsigned char smemRaw[];
    GroupSmem &sm = *reinterpret_cast<GroupSmem *>(smemRaw);
    __shared__ int warpSums[kGroupThreads / 32];
    const int side = blockIdx.x;
    const uint64_t *keys = side ? keyB : keyA;
    const int ob = side ? orderBitsB : orderBitsA, endBit = side ? endBitB : endBitA;
    int *uq = side ? uqB : uqA, *ct = side ? ctB : ctA;
    unsigned long long k[kGroupItems];
    int v[kGroupItems];
    const unsigned long long pad = endBit >= 64 ? ~0ull : ((1ull << endBit) - 1);
    for (int j = 0; j < kGroupItems; ++j) {
        const int i = threadIdx.x * kGroupItems + j;
        if (i < K) {
            const uint64_t key = keys[i];
            k[j] = ((key >> 32) << ob) | (key & 0xFFFFFFFFull);
            v[j] = val[i];
        } else {
            k[j] = pad; // sorts after every real key (LSD radix sort is stable and these come last)
            v[j] = -1;
        }
    }
    GroupSort(sm.sort).Sort(k, v, faceOnly ? ob : 0, endBit);
    __syncthreads(); // the sort storage is reused below
    int flags = 0;
    int prevFace = -1;
    const int i0 = threadIdx.x * kGroupItems;
    __shared__ int lastFace[kGroupThreads]; // face of each thread's last item, for its successor
    lastFace[threadIdx.x] = (int)(k[kGroupItems - 1] >> ob);
    __syncthreads();
    prevFace = threadIdx.x > 0 ? lastFace[threadIdx.x - 1] : -1;
    for (int j = 0; j < kGroupItems; ++j) {
        const int i = i0 + j;
        const int face = (int)(k[j] >> ob);
        if (i < K) {
            pairIdx[(size_t)side * K + i] = v[j];
            flags += (i == 0 || face != prevFace) ? 1 : 0;
        }
        prevFace = face;
    }
    // run index of each face start
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int incl = flags;
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o)
            incl += t;
    }
    if (lane == 31)
        warpSums[w] = incl;
    __syncthreads();
    int run = incl - flags, total = 0;
    for (int q = 0; q < kGroupThreads / 32; ++q) {
        run += q < w ? warpSums[q] : 0;
        total += warpSums[q];
    }
    prevFace = threadIdx.x > 0 ? lastFace[threadIdx.x - 1] : -1;
    for (int j = 0; j < kGroupItems; ++j) {
        const int i = i0 + j;
        const int face = (int)(k[j] >> ob);
        if (i < K && (i == 0 || face != prevFace)) {
            uq[run] = face;
            sm.starts[run] = i;
            ++run;
        }
        prevFace = face;
    }
    if (threadIdx.x == 0)
        sm.starts[total] = K;
    __syncthreads();
    for (int r = threadIdx.x; r < total; r += kGroupThreads)
        ct[r] = sm.starts[r + 1] - sm.starts[r];
    if (threadIdx.x == 0)
        runCount[side] = (unsigned int)total;
}

// ---- adjoint of the combine, its combinatorics held fixed --------------------------------------------
// An appended vertex is the representative of its weld class, a segment end built by CONSTRUCT_INTERSECTION
// (tri_tri_intersect.c:285-356) as x = b - a (b - o), a = ((b - r).N) / ((b - o).N), with b, r, o three of
// the pair's six vertices and N the normal cross(P1 - P0, P2 - P0) of the first triangle or
// cross(P3 - P5, P4 - P5) of the second. With u = b - r, w = b - o, D = w.N and c = -(g.w) / D for the
// upstream gradient g:  dL/db = (1 - a)(g + cN), dL/dr = -cN, dL/do = a (g + cN), dL/dN = c (u - a w);
// dL/dN reaches the triangle's vertices through the cross product. Input vertices keep their gradient.
__device__ __forceinline__ void atomic_add3(double *p, d3 v)
{
    atomicAdd(p, v.x);
    atomicAdd(p + 1, v.y);
    atomicAdd(p + 2, v.z);
}

__global__ void k_adjoint(size_t nv, int nvA, int nvB, const double *__restrict__ grad, const int *__restrict__ newSrc,
                          const uint32_t *__restrict__ pairAB, const uint32_t *__restrict__ pairPerm, MeshDev A,
                          MeshDev B, double *gradA, double *gradB)
{
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= nv)
        return;
    const d3 g = mk(grad[3 * i], grad[3 * i + 1], grad[3 * i + 2]);
    if (i < (size_t)nvA) {
        atomic_add3(gradA + 3 * i, g);
        return;
    }
    if (i < (size_t)nvA + nvB) {
        atomic_add3(gradB + 3 * (i - nvA), g);
        return;
    }
    const int src = newSrc[i - nvA - nvB];
    const int j = src >> 1, end = src & 1;
    const uint32_t code = pairPerm[j];
    int slot[6];
    for (int k = 0; k < 6; ++k)
        slot[k] = (int)((code >> (3 * k)) & 7u);
    const int which = (int)((code >> 18) & 3u);
    // vertex of each physical slot: 0..2 the first triangle, 3..5 the second
    const uint32_t ta = pairAB[2 * (size_t)j], tb = pairAB[2 * (size_t)j + 1];
    int vid[6];
    d3 P[6];
    for (int k = 0; k < 3; ++k) {
        vid[k] = (int)A.t[3 * (size_t)ta + k];
        vid[3 + k] = (int)B.t[3 * (size_t)tb + k];
        P[k] = mk(A.v[3 * (size_t)vid[k]], A.v[3 * (size_t)vid[k] + 1], A.v[3 * (size_t)vid[k] + 2]);
        P[3 + k] = mk(B.v[3 * (size_t)vid[3 + k]], B.v[3 * (size_t)vid[3 + k] + 1], B.v[3 * (size_t)vid[3 + k] + 2]);
    }
    const int p1 = slot[0], q1 = slot[1], r1 = slot[2], p2 = slot[3], q2 = slot[4], r2 = slot[5];
    int sb, sr, so, tri; // base, ref, other, normal of triangle 0 (first) or 1 (second)
    if (end == 0) {
        const bool on1 = which == 0 || which == 2;
        sb = on1 ? p1 : p2;
        sr = on1 ? p2 : p1;
        so = on1 ? r1 : q2;
        tri = on1 ? 1 : 0;
    } else {
        const bool on2 = which <= 1;
        sb = on2 ? p2 : p1;
        sr = on2 ? p1 : p2;
        so = on2 ? r2 : q1;
        tri = on2 ? 0 : 1;
    }
    const d3 e1 = tri == 0 ? P[1] - P[0] : P[3] - P[5];
    const d3 e2 = tri == 0 ? P[2] - P[0] : P[4] - P[5];
    const d3 N = cross(e1, e2);
    const d3 u = P[sb] - P[sr], w = P[sb] - P[so];
    const double D = dot(w, N);
    if (D == 0.0)
        return; // a degenerate construction the forward pass could not have produced finitely
    const double al = dot(u, N) / D;
    const double c = -dot(g, w) / D;
    const d3 gc = g + scale(c, N);
    d3 gP[6];
    for (int k = 0; k < 6; ++k)
        gP[k] = mk(0, 0, 0);
    gP[sb] = gP[sb] + scale(1.0 - al, gc);
    gP[sr] = gP[sr] - scale(c, N);
    gP[so] = gP[so] + scale(al, gc);
    const d3 gN = scale(c, u - scale(al, w));
    const d3 ge1 = cross(e2, gN), ge2 = cross(gN, e1); // N = e1 x e2
    if (tri == 0) {
        gP[1] = gP[1] + ge1;
        gP[2] = gP[2] + ge2;
        gP[0] = gP[0] - (ge1 + ge2);
    } else {
        gP[3] = gP[3] + ge1;
        gP[4] = gP[4] + ge2;
        gP[5] = gP[5] - (ge1 + ge2);
    }
    for (int k = 0; k < 3; ++k) {
        atomic_add3(gradA + 3 * (size_t)vid[k], gP[k]);
        atomic_add3(gradB + 3 * (size_t)vid[3 + k], gP[3 + k]);
    }
}

__global__ void k_face_table(int FA, int FB, const int *__restrict__ uniqA, const int *__restrict__ cntA,
                             const int *__restrict__ uniqB, const int *__restrict__ cntB, int *faceSide,
                             int *faceTri, int *faceCnt)
{
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= FA + FB)
        return;
    if (f < FA) {
        faceSide[f] = 0;
        faceTri[f] = uniqA[f];
        faceCnt[f] = cntA[f];
    } else {
        faceSide[f] = 1;
        faceTri[f] = uniqB[f - FA];
        faceCnt[f] = cntB[f - FA];
    }
}

__global__ void k_face_status(int nFaces, const int *__restrict__ faceSide, const int *__restrict__ status,
                              int *firstFail)
{
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nFaces)
        return;
    int st = status[f];
    if (st == 0)
        return;
    if (st == 3)
        atomicMin(firstFail + 2, f);
    else
        atomicMin(firstFail + faceSide[f], f);
}

// 1 for the uncut triangles the reference keeps: not cut, and not past the mesh's truncation point
__global__ void k_not_flag(int n, const int *__restrict__ flag, int *out, const int *__restrict__ truncOcc)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        out[i] = (flag[i] || i > *truncOcc / 3) ? 0 : 1;
}

// Truncation point of a mesh that holds a directed edge twice: every uncut triangle's edges in insertion
// order (occurrence 3 i + k) into a table keeping the first occurrence of each half-edge; the first
// occurrence that finds its half-edge already taken is where the reference's insertion fails.
__global__ void k_trunc_insert(int nt, const uint32_t *__restrict__ t, const int *__restrict__ cut, uint64_t *keys,
                               int *vals, uint32_t mask)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt || cut[i])
        return;
    for (int k = 0; k < 3; ++k)
        u64map_insert_min(keys, vals, mask, he_key(t[3 * (size_t)i + k], t[3 * (size_t)i + (k + 1) % 3]), 3 * i + k);
}

__global__ void k_trunc_find(int nt, const uint32_t *__restrict__ t, const int *__restrict__ cut,
                             const uint64_t *__restrict__ keys, const int *__restrict__ vals, uint32_t mask,
                             int *truncOcc)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt || cut[i])
        return;
    for (int k = 0; k < 3; ++k) {
        const int occ = 3 * i + k;
        if (u64map_find(keys, vals, mask, he_key(t[3 * (size_t)i + k], t[3 * (size_t)i + (k + 1) % 3])) < occ)
            atomicMin(truncOcc, occ);
    }
}

__global__ void k_tri_mesh(int nTri, int uncutA, int uncutB, int retriA, int8_t *triMesh, int8_t *isUncut)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nTri)
        return;
    bool first = t < uncutA || (t >= uncutA + uncutB && t < uncutA + uncutB + retriA);
    triMesh[t] = first ? 0 : 1;
    isUncut[t] = t < uncutA + uncutB ? 1 : 0;
}

__global__ void k_cand_pairs(int n, const uint64_t *__restrict__ cand, int nB, uint32_t *out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    uint64_t key = cand[i];
    uint32_t a = (uint32_t)(key / (uint64_t)nB);
    out[2 * (size_t)i] = a;
    out[2 * (size_t)i + 1] = (uint32_t)(key - (uint64_t)a * (uint64_t)nB);
}

} // namespace sbg

using namespace sbg;

// ---------------------------------------------------------------------------------------------------
// boolean handle
// ---------------------------------------------------------------------------------------------------
struct sb_boolean {
    const sb_mesh *first = nullptr, *second = nullptr;
    sb_options opts;
    cudaStream_t s = nullptr;
    // working and result buffers
    DevBuf cand, isect, faces, scratch, cut, weld, arr, groups, res, cub, small, trunc, sides, order, flood;
    unsigned int candCap = 0;
    bool combined = false;
    sb_status status = SB_ERR_NOT_COMBINED;
    sb_stats stats;
    // device views kept for fetch / dumps
    uint64_t *d_cand = nullptr;
    int C = 0, K = 0;
    uint32_t *d_pairAB = nullptr;
    double *d_segK = nullptr;
    // for the adjoint: each intersecting pair's construction record, and the source (2 x pair + segment end)
    // of every appended vertex
    uint32_t *d_pairPerm = nullptr;
    int *d_newSrc = nullptr;
    int newBase = 0;
    double *d_newV = nullptr;
    size_t nNewV = 0;
    uint32_t *d_newT = nullptr;
    int nTri = 0;
    int8_t *d_label = nullptr, *d_triMesh = nullptr;
    uint32_t *d_fetch[3] = {nullptr, nullptr, nullptr};
    size_t nFetch[3] = {0, 0, 0};
    cudaEvent_t ev[10];
    cudaStream_t side = nullptr;     // second stream for preparing the two meshes concurrently
    cudaEvent_t sideDone = nullptr;
    cudaEvent_t orderDone = nullptr; // the cut faces' processing order, computed on `side`
    cudaEvent_t retriDone = nullptr; // the re-triangulated triangles' numbering, computed on `side`
    bool evInit = false;
    char *mail = nullptr; // pinned mailbox: small reads [0, kMailRead), constant uploads after it
    // results staged in page-locked host memory (sb_options.stage_results): the three fetches, the vertices
    struct Staged {
        void *ptr = nullptr;
        size_t count = 0;
    } staged[4];
    cudaStream_t stage = nullptr; // copy stream of the vertex staging
    cudaEvent_t stageEv = nullptr;
    bool staging = false;         // a copy to the host is in flight on `stage`
};

constexpr size_t kMailRead = kMailBytes - 64;

namespace {

// waits for the vertex staging copy, if one is in flight
cudaError_t staged_wait(sb_boolean *b)
{
    if (!b->staging)
        return cudaSuccess;
    b->staging = false;
    return cudaStreamSynchronize(b->stage);
}

// releases the staged buffers nobody took
void staged_release(sb_boolean *b)
{
    for (auto &x : b->staged) {
        if (x.ptr)
            sb_host_free(x.ptr);
        x = sb_boolean::Staged{};
    }
}

template <class F> sb_status guarded(F &&f)
{
    try {
        return f();
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return SB_ERR_INVALID;
    }
}

// CUB wrappers: query, grow the handle's temp buffer, run
template <class Call> cudaError_t cub_run(sb_boolean *b, Call &&call)
{
    size_t need = 0;
    cudaError_t e = call(nullptr, need);
    if (e != cudaSuccess)
        return e;
    e = b->cub.ensure(need);
    if (e != cudaSuccess)
        return e;
    size_t have = b->cub.bytes;
    return call(b->cub.ptr, have);
}

// Small device-to-host reads through the boolean's pinned mailbox: queued on its stream, one synchronisation
// for all of them, then copied out. (A pageable destination would take the driver's staging path, which
// serialises the streams of concurrent booleans.)
class Readback {
public:
    explicit Readback(sb_boolean *b) : b_(b) {}
    cudaError_t add(void *dst, const void *src, size_t bytes)
    {
        const size_t at = (used_ + 7) & ~(size_t)7;
        if (at + bytes > kMailRead || n_ == kItems)
            return cudaErrorInvalidValue;
        const cudaError_t e = cudaMemcpyAsync(b_->mail + at, src, bytes, cudaMemcpyDeviceToHost, b_->s);
        if (e != cudaSuccess)
            return e;
        items_[n_++] = Item{dst, at, bytes};
        used_ = at + bytes;
        return cudaSuccess;
    }
    cudaError_t sync()
    {
        const cudaError_t e = cudaStreamSynchronize(b_->s);
        if (e != cudaSuccess)
            return e;
        for (int i = 0; i < n_; ++i)
            std::memcpy(items_[i].dst, b_->mail + items_[i].at, items_[i].bytes);
        n_ = 0;
        used_ = 0;
        return cudaSuccess;
    }

private:
    struct Item {
        void *dst;
        size_t at, bytes;
    };
    static constexpr int kItems = 16;
    sb_boolean *b_;
    Item items_[kItems];
    int n_ = 0;
    size_t used_ = 0;
};

sb_status read_back(sb_boolean *b, void *dst, const void *src, size_t bytes)
{
    Readback rb(b);
    SB_CUDA_CHECK(rb.add(dst, src, bytes));
    SB_CUDA_CHECK(rb.sync());
    return SB_OK;
}

int end_bit_for(uint64_t maxValue)
{
    int bits = 1;
    while (bits < 64 && (maxValue >> bits) != 0)
        ++bits;
    return bits;
}

sb_status combine_impl(sb_boolean *b)
{
    cudaStream_t s = b->s;
    const MeshDev &A = b->first->d;
    const MeshDev &B = b->second->d;
    const bool fp64 = b->opts.precision == SB_PRECISION_FP64;
    const double factor = (double)b->opts.weld_factor;
    sb_stats &st = b->stats;
    std::memset(&st, 0, sizeof st);
    b->combined = false;
    SB_CUDA_CHECK(staged_wait(b));
    staged_release(b);
    for (int k = 0; k < 3; ++k) {
        b->d_fetch[k] = nullptr;
        b->nFetch[k] = 0;
    }
    if (!b->evInit) {
        for (auto &e : b->ev)
            SB_CUDA_CHECK(cudaEventCreate(&e));
        b->evInit = true;
    }
    // the second stream (work that runs beside the main chain) and its hand-over events
    if (!b->side) {
        SB_CUDA_CHECK(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking));
        SB_CUDA_CHECK(cudaEventCreateWithFlags(&b->sideDone, cudaEventDisableTiming));
    }
    if (!b->orderDone)
        SB_CUDA_CHECK(cudaEventCreateWithFlags(&b->orderDone, cudaEventDisableTiming));
    if (!b->retriDone)
        SB_CUDA_CHECK(cudaEventCreateWithFlags(&b->retriDone, cudaEventDisableTiming));
    // the meshes may have been prepared on other streams
    for (const sb_mesh *cm : {b->first, b->second})
        if (cm->readyEv)
            SB_CUDA_CHECK(cudaStreamWaitEvent(s, cm->readyEv, 0));
    SB_CUDA_CHECK(cudaEventRecord(b->ev[0], s));

    // small device block: [0..7] stats u64, [8..] counters, firstFail, scalars
    SB_CUDA_CHECK(b->small.ensure(4096));
    unsigned long long *d_stats = b->small.as<unsigned long long>();
    unsigned int *d_count = reinterpret_cast<unsigned int *>(b->small.as<char>() + 128);
    unsigned int *d_counters = reinterpret_cast<unsigned int *>(b->small.as<char>() + 256);
    int *d_firstFail = reinterpret_cast<int *>(b->small.as<char>() + 512);
    SB_CUDA_CHECK(cudaMemsetAsync(b->small.ptr, 0, 1024, s));

    const int nA = A.nt, nB = B.nt;
    // directed edges held more than once per input mesh (1: unknown, treated as present)
    int adjDup[2] = {1, 1};
    int *d_truncOcc = reinterpret_cast<int *>(b->small.as<char>() + 640);
    SB_CUDA_CHECK(cudaMemsetAsync(d_truncOcc, 0x7F, 2 * sizeof(int), s)); // no truncation
    // ---------------- broad phase ----------------
    if (b->candCap == 0)
        b->candCap = (unsigned int)std::max<size_t>(4096, 4 * ((size_t)nA + (size_t)nB));
    unsigned int C = 0;
    for (int attempt = 0; attempt < 3; ++attempt) {
        Carve c;
        size_t o_raw = c.take<uint64_t>(b->candCap);
        size_t o_srt = c.take<uint64_t>(b->candCap);
        size_t o_hit = c.take<uint8_t>(b->candCap);
        size_t o_seg = c.take<double>((size_t)b->candCap * 6);
        size_t o_sel = c.take<int>(b->candCap);
        c.take<uint32_t>(b->candCap); // per-candidate construction record
        SB_CUDA_CHECK(b->cand.ensure(c.off));
        (void)o_hit;
        (void)o_seg;
        (void)o_sel;
        SB_CUDA_CHECK(cudaMemsetAsync(d_count, 0, sizeof(unsigned int), s));
        SB_CUDA_CHECK(cudaMemsetAsync(d_stats, 0, 8 * sizeof(unsigned long long), s));
        Readback rb(b);
        if (attempt == 0 && A.adj && B.adj) { // read with the candidate count below
            SB_CUDA_CHECK(rb.add(adjDup, A.adjDup, sizeof(int)));
            SB_CUDA_CHECK(rb.add(adjDup + 1, B.adjDup, sizeof(int)));
        }
        launch_broad(fp64, A, B, reinterpret_cast<uint64_t *>(b->cand.as<char>() + o_raw), d_count, b->candCap,
                     d_stats, s);
        SB_CUDA_CHECK(cudaGetLastError());
        SB_CUDA_CHECK(rb.add(&C, d_count, sizeof C));
        SB_CUDA_CHECK(rb.sync());
        if (C <= b->candCap)
            break;
        b->candCap = C + C / 4 + 1024;
    }
    Carve cc;
    size_t o_raw = cc.take<uint64_t>(b->candCap);
    size_t o_srt = cc.take<uint64_t>(b->candCap);
    size_t o_hit = cc.take<uint8_t>(b->candCap);
    size_t o_seg = cc.take<double>((size_t)b->candCap * 6);
    size_t o_sel = cc.take<int>(b->candCap);
    size_t o_perm = cc.take<uint32_t>(b->candCap);
    uint64_t *candRaw = reinterpret_cast<uint64_t *>(b->cand.as<char>() + o_raw);
    uint64_t *candSorted = reinterpret_cast<uint64_t *>(b->cand.as<char>() + o_srt); // unused, see below
    uint8_t *hit = reinterpret_cast<uint8_t *>(b->cand.as<char>() + o_hit);
    double *seg = reinterpret_cast<double *>(b->cand.as<char>() + o_seg);
    int *sel = reinterpret_cast<int *>(b->cand.as<char>() + o_sel);
    uint32_t *perm = reinterpret_cast<uint32_t *>(b->cand.as<char>() + o_perm);
    // Candidates stay in emission order: every later ordering is by unique keys (face, the other triangle's
    // leaf position), so the result does not depend on it.
    (void)candSorted;
    candSorted = candRaw;
    b->C = (int)C;
    b->d_cand = candSorted;
    st.candidate_pairs = C;
    SB_CUDA_CHECK(cudaEventRecord(b->ev[1], s));

    // ---------------- narrow phase ----------------
    launch_narrow(fp64, A, B, candSorted, (int)C, hit, seg, perm, d_stats, s);
    SB_CUDA_CHECK(cudaGetLastError());
    if (C > 0)
        SB_CUDA_CHECK(cub_run(b, [&](void *tmp, size_t &bytes) {
            return cub::DeviceSelect::Flagged(tmp, bytes, thrust::counting_iterator<int>(0), hit, sel,
                                              d_count + 1, (int)C, s);
        }));
    // The count of intersecting pairs stays on the device until the faces are counted (a host round trip
    // fewer), the candidate count bounding the buffers it would size: the one-block grouping takes the count
    // from the device, and only a count beyond its reach is grouped device-wide once read.
    constexpr unsigned int kDeferMax = 1u << 20;
    unsigned int K = 0;
    const bool deferK = C > 0 && C <= kDeferMax;
    if (C > 0 && !deferK) {
        sb_status r = read_back(b, &K, d_count + 1, sizeof K);
        if (r != SB_OK)
            return r;
    }
    const unsigned int Kcap = deferK ? C : K; // buffer sizes and grids
    const unsigned int *dK = deferK ? d_count + 1 : nullptr;
    SB_CUDA_CHECK(cudaEventRecord(b->ev[2], s));

    // ---------------- face lists ----------------
    Carve ci;
    size_t o_keyA = ci.take<uint64_t>(Kcap + 1), o_keyB = ci.take<uint64_t>(Kcap + 1);
    size_t o_keyAs = ci.take<uint64_t>(Kcap + 1), o_keyBs = ci.take<uint64_t>(Kcap + 1);
    size_t o_val = ci.take<int>(Kcap + 1), o_pidx = ci.take<int>(2 * (size_t)Kcap + 2);
    size_t o_segK = ci.take<double>(6 * (size_t)Kcap + 6), o_ab = ci.take<uint32_t>(2 * (size_t)Kcap + 2);
    size_t o_pp = ci.take<uint32_t>((size_t)Kcap + 1);
    size_t o_hiA = ci.take<int>(Kcap + 1), o_hiB = ci.take<int>(Kcap + 1);
    size_t o_uqA = ci.take<int>(Kcap + 1), o_uqB = ci.take<int>(Kcap + 1);
    size_t o_ctA = ci.take<int>(Kcap + 1), o_ctB = ci.take<int>(Kcap + 1);
    SB_CUDA_CHECK(b->isect.ensure(ci.off));
    char *ib = b->isect.as<char>();
    uint64_t *keyA = (uint64_t *)(ib + o_keyA), *keyB = (uint64_t *)(ib + o_keyB);
    uint64_t *keyAs = (uint64_t *)(ib + o_keyAs), *keyBs = (uint64_t *)(ib + o_keyBs);
    int *val = (int *)(ib + o_val), *pairIdx = (int *)(ib + o_pidx);
    double *segK = (double *)(ib + o_segK);
    uint32_t *pairAB = (uint32_t *)(ib + o_ab);
    int *hiA = (int *)(ib + o_hiA), *hiB = (int *)(ib + o_hiB);
    int *uqA = (int *)(ib + o_uqA), *uqB = (int *)(ib + o_uqB), *ctA = (int *)(ib + o_ctA), *ctB = (int *)(ib + o_ctB);
    b->d_pairAB = pairAB;
    uint32_t *pairPerm = (uint32_t *)(ib + o_pp);
    b->d_pairPerm = pairPerm;
    b->d_segK = segK;
    // The leaf orders may still be building on the meshes' second streams (they overlap the broad and narrow
    // phases). Nothing before the re-triangulation needs them: the pairs are grouped by face, the faces
    // counted and their capacities sized, and the arrangement's uncut parts prepared first; the stream waits
    // for the leaf orders only before the pairs of each face are put in the reference's order.
    auto waitRanks = [&]() -> sb_status {
        for (const sb_mesh *cm : {b->first, b->second})
            if (cm->rankPending && cm->aux)
                SB_CUDA_CHECK(cudaStreamWaitEvent(s, cm->auxJoin, 0));
        return SB_OK;
    };
    auto rankResults = [&]() -> sb_status {
        for (const sb_mesh *cm : {b->first, b->second}) {
            const sb_status r = reference_rank_result(const_cast<sb_mesh *>(cm));
            if (r != SB_OK)
                return r;
        }
        return SB_OK;
    };
    const bool useRank = b->opts.order == SB_ORDER_REFERENCE && A.rankValid && B.rankValid;
    int FA = 0, FB = 0;
    if (Kcap > 0) {
        SB_COUNT(k_pair_keys)<<<blocks(Kcap, 256), 256, 0, s>>>((int)Kcap, dK, sel, candSorted, nB, nullptr, nullptr,
                                                      seg, perm, keyA, keyB, val, segK, pairAB, pairPerm);
        // device-wide grouping (the count K known on the host)
        auto groupDeviceWide = [&]() -> sb_status {
            SB_CUDA_CHECK(cub_run(b, [&](void *tmp, size_t &bytes) {
                return cub::DeviceRadixSort::SortPairs(tmp, bytes, keyA, keyAs, val, pairIdx, (int)K, useRank ? 32 : 0,
                                                       64, s); // by face alone when the pair order follows
            }));
            SB_CUDA_CHECK(cub_run(b, [&](void *tmp, size_t &bytes) {
                return cub::DeviceRadixSort::SortPairs(tmp, bytes, keyB, keyBs, val, pairIdx + K, (int)K,
                                                       useRank ? 32 : 0, 64, s);
            }));
            SB_COUNT(k_hi32)<<<blocks(K, 256), 256, 0, s>>>((int)K, keyAs, hiA);
            SB_COUNT(k_hi32)<<<blocks(K, 256), 256, 0, s>>>((int)K, keyBs, hiB);
            SB_CUDA_CHECK(cub_run(b, [&](void *tmp, size_t &bytes) {
                return cub::DeviceRunLengthEncode::Encode(tmp, bytes, hiA, uqA, ctA, d_count + 2, (int)K, s);
            }));
            SB_CUDA_CHECK(cub_run(b, [&](void *tmp, size_t &bytes) {
                return cub::DeviceRunLengthEncode::Encode(tmp, bytes, hiB, uqB, ctB, d_count + 3, (int)K, s);
            }));
            return SB_OK;
        };
        if (deferK || Kcap <= (unsigned int)kGroupMax) {
            const int obA = end_bit_for((uint64_t)std::max(nB, 1)), obB = end_bit_for((uint64_t)std::max(nA, 1));
            const int ebA = obA + end_bit_for((uint64_t)std::max(nA, 1)), ebB = obB + end_bit_for((uint64_t)std::max(nB, 1));
            static std::once_flag smemOnce;
            std::call_once(smemOnce, [] {
                cudaFuncSetAttribute(k_face_group, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(GroupSmem));
            });
            SB_COUNT(k_face_group)<<<2, kGroupThreads, sizeof(GroupSmem), s>>>(
                (int)Kcap, dK, keyA, keyB, val, obA, obB, ebA, ebB, useRank, pairIdx, uqA, ctA, uqB, ctB, d_count + 2);
        } else {
            const sb_status r = groupDeviceWide();
            if (r != SB_OK)
                return r;
        }
        unsigned int runs[2];
        {
            Readback rb(b);
            SB_CUDA_CHECK(rb.add(runs, d_count + 2, sizeof runs));
            if (deferK)
                SB_CUDA_CHECK(rb.add(&K, d_count + 1, sizeof K));
            SB_CUDA_CHECK(rb.sync());
        }
        if (deferK && K > (unsigned int)kGroupMax) { // the one-block grouping left them
            const sb_status r = groupDeviceWide();
            if (r != SB_OK)
                return r;
            Readback rb(b);
            SB_CUDA_CHECK(rb.add(runs, d_count + 2, sizeof runs));
            SB_CUDA_CHECK(rb.sync());
        }
        FA = (int)runs[0];
        FB = (int)runs[1];
    }
    b->K = (int)K;
    st.intersecting_pairs = K;
    const int nFaces = FA + FB;
    st.cut_faces_first = FA;
    st.cut_faces_second = FB;

    // ---------------- per-face capacities and re-triangulation ----------------
    Carve cf;
    size_t o_side = cf.take<int>(nFaces + 1), o_tri = cf.take<int>(nFaces + 1), o_cnt = cf.take<int>(nFaces + 1);
    size_t o_beg = cf.take<int>(nFaces + 1), o_sb = cf.take<unsigned long long>(nFaces + 1);
    size_t o_so = cf.take<unsigned long long>(nFaces + 1);
    size_t o_pc = cf.take<int>(nFaces + 1), o_tc = cf.take<int>(nFaces + 1), o_ec = cf.take<int>(nFaces + 1);
    size_t o_po = cf.take<int>(nFaces + 1), o_to = cf.take<int>(nFaces + 1), o_eo = cf.take<int>(nFaces + 1);
    size_t o_fst = cf.take<int>(nFaces + 1), o_fnp = cf.take<int>(nFaces + 1), o_fnt = cf.take<int>(nFaces + 1);
    size_t o_fne = cf.take<int>(nFaces + 1), o_rr = cf.take<int>(nFaces + 1);
    size_t o_frm = cf.take<double>(6 * ((size_t)nFaces + 1));
    SB_CUDA_CHECK(b->faces.ensure(cf.off));
    char *fb = b->faces.as<char>();
    int *faceSide = (int *)(fb + o_side), *faceTri = (int *)(fb + o_tri), *faceCnt = (int *)(fb + o_cnt);
    int *faceBegin = (int *)(fb + o_beg);
    unsigned long long *scratchBytes = (unsigned long long *)(fb + o_sb), *scratchOff = (unsigned long long *)(fb + o_so);
    int *ptCap = (int *)(fb + o_pc), *triCapA = (int *)(fb + o_tc), *edgeCap = (int *)(fb + o_ec);
    int *ptOff = (int *)(fb + o_po), *triOff = (int *)(fb + o_to), *edgeOff = (int *)(fb + o_eo);
    int *faceStatus = (int *)(fb + o_fst), *faceNpts = (int *)(fb + o_fnp), *faceNtris = (int *)(fb + o_fnt);
    int *faceNedges = (int *)(fb + o_fne), *retriRank = (int *)(fb + o_rr);
    double *faceFrames = (double *)(fb + o_frm);
    SB_CUDA_CHECK(cudaMemsetAsync(fb, 0, cf.off, s));
    long long totals[4] = {0, 0, 0, 0};
    int *faceRank = nullptr, *faceByRank = nullptr, *ptRef = nullptr, *edgeRef = nullptr, *retriRef = nullptr;
    int *rankTmp[3] = {nullptr, nullptr, nullptr}, *rankTot = nullptr;
    bool orderPending = false;
    FaceOrderArgs fo;   // the faces' processing order (second stream), set up with the face capacities
    RankScanArgs ra;
    int *rankPart2 = nullptr;
    char *ob = nullptr;
    size_t o_fks = 0, o_fvs = 0;
    if (nFaces > 0) {
        if (nFaces <= kFaceLayoutBlockMax) {
            launch_face_layout(FA, FB, uqA, ctA, uqB, ctB, faceSide, faceTri, faceCnt, faceBegin, scratchOff, ptCap,
                               ptOff, triCapA, triOff, edgeCap, edgeOff, s);
        } else {
            SB_COUNT(k_face_table)<<<blocks(nFaces, 256), 256, 0, s>>>(FA, FB, uqA, ctA, uqB, ctB, faceSide, faceTri,
                                                                       faceCnt);
            SB_CUDA_CHECK(cub_run(b, [&](void *tmp, size_t &bytes) {
                return cub::DeviceScan::ExclusiveSum(tmp, bytes, faceCnt, faceBegin, nFaces + 1, s);
            }));
            launch_face_sizes(nFaces, faceBegin, scratchBytes, ptCap, triCapA, edgeCap, s);
            SB_CUDA_CHECK(cub_run(b, [&](void *tmp, size_t &bytes) {
                return cub::DeviceScan::ExclusiveSum(tmp, bytes, scratchBytes, scratchOff, nFaces + 1, s);
            }));
            SB_CUDA_CHECK(cub_run(b, [&](void *tmp, size_t &bytes) {
                return cub::DeviceScan::ExclusiveSum(tmp, bytes, ptCap, ptOff, nFaces + 1, s);
            }));
            SB_CUDA_CHECK(cub_run(b, [&](void *tmp, size_t &bytes) {
                return cub::DeviceScan::ExclusiveSum(tmp, bytes, triCapA, triOff, nFaces + 1, s);
            }));
            SB_CUDA_CHECK(cub_run(b, [&](void *tmp, size_t &bytes) {
                return cub::DeviceScan::ExclusiveSum(tmp, bytes, edgeCap, edgeOff, nFaces + 1, s);
            }));
        }
        launch_face_frames(nFaces, faceSide, faceTri, A, B, faceFrames, s); // needs no leaf order
        // the reference's processing order of the cut faces: each face keyed by its first pair's place in the
        // tree traversal, sorted, then ordered like the context map iterates them
        Carve co;
        const size_t o_fk = co.take<unsigned long long>(nFaces);
        o_fks = co.take<unsigned long long>(nFaces);
        const size_t o_fv = co.take<int>(nFaces);
        o_fvs = co.take<int>(nFaces);
        const size_t o_fr = co.take<int>(nFaces + 1), o_fbr = co.take<int>(nFaces + 1);
        const size_t o_ik = co.take<uint32_t>(nFaces + 1);
        const size_t o_hA = co.take<int>(hash_scratch_ints(FA)), o_hB = co.take<int>(hash_scratch_ints(FB));
        const size_t o_pr = co.take<int>(nFaces + 1), o_er = co.take<int>(nFaces + 1), o_rr2 = co.take<int>(nFaces + 1);
        const size_t o_t0 = co.take<int>(nFaces + 1), o_t1 = co.take<int>(nFaces + 1), o_t2 = co.take<int>(nFaces + 1);
        const size_t o_tot = co.take<int>(8), o_part = co.take<int>(3 * 1024), o_part2 = co.take<int>(3 * 1024);
        SB_CUDA_CHECK(b->order.ensure(co.off));
        ob = b->order.as<char>();
        fo.nFaces = nFaces;
        fo.FA = FA;
        fo.FB = FB;
        fo.faceTri = faceTri;
        fo.faceBegin = faceBegin;
        fo.pairIdx = pairIdx;
        fo.pairAB = pairAB;
        fo.A = A;
        fo.B = B;
        fo.exact = useRank && A.tnode && B.tnode ? 1 : 0;
        fo.key = (unsigned long long *)(ob + o_fk);
        fo.val = (int *)(ob + o_fv);
        fo.sortedVal = (const int *)(ob + o_fvs);
        fo.sortedOut = (int *)(ob + o_fvs);
        fo.blockSort = face_ctx_block_sort(FA, FB) ? 1 : 0;
        fo.faceRank = (int *)(ob + o_fr);
        fo.faceByRank = (int *)(ob + o_fbr);
        fo.insKeys = (uint32_t *)(ob + o_ik);
        fo.hs[0] = hash_scratch_at((int *)(ob + o_hA), FA);
        fo.hs[1] = hash_scratch_at((int *)(ob + o_hB), FB);
        fo.overflow = d_counters + kCntCount; // spare counter slot past the assembly's
        faceRank = fo.faceRank;
        faceByRank = fo.faceByRank;
        ptRef = (int *)(ob + o_pr);
        edgeRef = (int *)(ob + o_er);
        retriRef = (int *)(ob + o_rr2);
        rankTmp[0] = (int *)(ob + o_t0);
        rankTmp[1] = (int *)(ob + o_t1);
        rankTmp[2] = (int *)(ob + o_t2);
        rankTot = (int *)(ob + o_tot);
        std::memset(&ra, 0, sizeof ra);
        ra.n = nFaces;
        ra.FA = FA;
        ra.count = 2;
        ra.faceByRank = faceByRank;
        ra.faceRank = faceRank;
        ra.vals[0] = ptCap;
        ra.vals[1] = edgeCap;
        ra.out[0] = ptRef;
        ra.out[1] = edgeRef;
        ra.tmp[0] = rankTmp[0];
        ra.tmp[1] = rankTmp[1];
        ra.tot[0] = rankTot;
        ra.tot[1] = rankTot + 2;
        ra.part = (int *)(ob + o_part);
        rankPart2 = (int *)(ob + o_part2); // its own: the triangles' numbering may overlap this scan
        // The totals follow from the pair count without a read-back: every intersecting pair cuts one face of
        // each mesh, so the faces' pair counts sum to 2 K; a face of np pairs takes 2 np points, 2 np directed
        // edges and 32 np + 16 triangles. Its scratch is bounded by an affine function of np
        // (face_scratch_bound); the re-triangulation checks the bound per face.
        totals[0] = (long long)face_scratch_bound(nFaces, 2 * (long long)K);
        totals[1] = 4 * (long long)K;
        totals[2] = 64 * (long long)K + 16 * (long long)nFaces;
        totals[3] = 4 * (long long)K;
    }
    AsmArgs g;
    std::memset(&g, 0, sizeof g);
    g.nFaces = nFaces;
    g.faceSide = faceSide;
    g.faceTri = faceTri;
    // ---------------- arrangement ----------------
    Carve ca;
    size_t o_cA = ca.take<int>(nA + 1), o_cB = ca.take<int>(nB + 1), o_nA = ca.take<int>(nA + 1);
    size_t o_nB = ca.take<int>(nB + 1), o_rA = ca.take<int>(nA + 1), o_rB = ca.take<int>(nB + 1);
    SB_CUDA_CHECK(b->arr.ensure(ca.off));
    char *ab = b->arr.as<char>();
    g.cutA = (int *)(ab + o_cA);
    g.cutB = (int *)(ab + o_cB);
    int *notA = (int *)(ab + o_nA), *notB = (int *)(ab + o_nB);
    g.uncutRankA = (int *)(ab + o_rA);
    g.uncutRankB = (int *)(ab + o_rB);
    {
        Fills fl(s);
        fl.i32(g.cutA, nA + 1, 0);
        fl.i32(g.cutB, nB + 1, 0);
        fl.i32(notA, nA + 1, 0);
        fl.i32(notB, nB + 1, 0);
        fl.launch();
    }
    launch_mark_cut(g, s);
    g.truncOcc = d_truncOcc;
    for (int side = 0; side < 2; ++side) {
        // a mesh holding a directed edge twice: find where the reference's uncut-triangle insertion stops
        const MeshDev &M = side == 0 ? A : B;
        if (adjDup[side] == 0 || M.nt == 0)
            continue;
        const uint32_t cap = pow2_at_least(2 * 3 * (size_t)M.nt);
        SB_CUDA_CHECK(b->trunc.ensure((sizeof(uint64_t) + sizeof(int)) * (size_t)cap));
        uint64_t *tk = b->trunc.as<uint64_t>();
        int *tv = reinterpret_cast<int *>(tk + cap);
        SB_CUDA_CHECK(cudaMemsetAsync(tk, 0xFF, sizeof(uint64_t) * cap, s));
        SB_CUDA_CHECK(cudaMemsetAsync(tv, 0x7F, sizeof(int) * cap, s));
        const int *cutM = side == 0 ? g.cutA : g.cutB;
        SB_COUNT(k_trunc_insert)<<<blocks(M.nt, 256), 256, 0, s>>>(M.nt, M.t, cutM, tk, tv, cap - 1);
        SB_COUNT(k_trunc_find)<<<blocks(M.nt, 256), 256, 0, s>>>(M.nt, M.t, cutM, tk, tv, cap - 1, d_truncOcc + side);
    }
    if (nA > 0)
        SB_COUNT(k_not_flag)<<<blocks(nA, 256), 256, 0, s>>>(nA, g.cutA, notA, d_truncOcc);
    if (nB > 0)
        SB_COUNT(k_not_flag)<<<blocks(nB, 256), 256, 0, s>>>(nB, g.cutB, notB, d_truncOcc + 1);
    SB_CUDA_CHECK(cub_run(b, [&](void *tmp, size_t &bytes) {
        return cub::DeviceScan::ExclusiveSum(tmp, bytes, notA, g.uncutRankA, nA + 1, s);
    }));
    SB_CUDA_CHECK(cub_run(b, [&](void *tmp, size_t &bytes) {
        return cub::DeviceScan::ExclusiveSum(tmp, bytes, notB, g.uncutRankB, nB + 1, s);
    }));
    // the global weld's tables, filled while the leaf orders finish
    const size_t nSeq = (size_t)totals[1];
    const uint32_t weldCap = pow2_at_least(2 * nSeq + 2);
    Carve cw;
    size_t o_wo = cw.take<int>(weldCap), o_wm = cw.take<int>(weldCap), o_ps = cw.take<int>(nSeq + 1);
    size_t o_if = cw.take<int>(nSeq + 1), o_fr = cw.take<int>(nSeq + 1), o_sr = cw.take<int>(weldCap);
    size_t o_nsrc = cw.take<int>(nSeq + 1);
    SB_CUDA_CHECK(b->weld.ensure(cw.off));
    char *wb = b->weld.as<char>();
    g.weldOwner = (int *)(wb + o_wo);
    g.weldMin = (int *)(wb + o_wm);
    g.weldMask = weldCap - 1;
    g.pointSlot = (int *)(wb + o_ps);
    g.isFirst = (int *)(wb + o_if);
    g.firstRank = (int *)(wb + o_fr);
    g.slotRank = (int *)(wb + o_sr);
    g.newSrc = (int *)(wb + o_nsrc);
    b->d_newSrc = g.newSrc;
    b->newBase = A.nv + B.nv;
    {
        Fills fl(s);
        fl.i32(g.weldOwner, weldCap, -1);
        fl.i32(g.weldMin, weldCap, INT_MAX);
        fl.i32(g.isFirst, nSeq + 1, 0);
        fl.launch();
    }
    // from here on the leaf orders are needed
    {
        const sb_status r = waitRanks();
        if (r != SB_OK)
            return r;
    }
    if (nFaces > 0) {
        if (useRank)
            SB_COUNT(k_face_pair_order)<<<blocks(nFaces, 128), 128, 0, s>>>(nFaces, FA, faceBegin, pairIdx, pairAB,
                                                                          A.rank, B.rank);
        // the processing order runs on the second stream beside the re-triangulation (the weld waits for it)
        cudaStream_t so = b->side;
        SB_CUDA_CHECK(cudaEventRecord(b->sideDone, s));
        SB_CUDA_CHECK(cudaStreamWaitEvent(so, b->sideDone, 0));
        launch_face_keys(fo, so);
        if (!fo.blockSort) // else k_face_ctx sorts each mesh's faces in its own block
            SB_CUDA_CHECK(cub_run(b, [&](void *tmp, size_t &bytes) {
                return cub::DeviceRadixSort::SortPairs(tmp, bytes, fo.key, (unsigned long long *)(ob + o_fks), fo.val,
                                                       (int *)(ob + o_fvs), nFaces, 0, 64, so);
            }));
        launch_face_ctx(fo, so);
        launch_rank_scan(ra, so);
        SB_CUDA_CHECK(cudaEventRecord(b->orderDone, so));
        orderPending = true;
    }
    Carve cu;
    size_t o_cp = cu.take<d3>(totals[1] + 1), o_ck = cu.take<Key>(totals[1] + 1);
    size_t o_psrc = cu.take<int>(totals[1] + 1);
    size_t o_ft = cu.take<int>(3 * totals[2] + 3), o_fe = cu.take<int>(2 * totals[3] + 2);
    SB_CUDA_CHECK(b->cut.ensure(cu.off));
    SB_CUDA_CHECK(b->scratch.ensure((size_t)totals[0] + 256));
    d3 *cutPts = (d3 *)(b->cut.as<char>() + o_cp);
    Key *cutKeys = (Key *)(b->cut.as<char>() + o_ck);
    int *ptSrc = (int *)(b->cut.as<char>() + o_psrc);
    int *faceTris = (int *)(b->cut.as<char>() + o_ft);
    int *faceEdges = (int *)(b->cut.as<char>() + o_fe);
    if (nFaces > 0) {
        FaceArgs fa;
        fa.A = A;
        fa.B = B;
        fa.nFaces = nFaces;
        fa.faceSide = faceSide;
        fa.faceTri = faceTri;
        fa.faceBegin = faceBegin;
        fa.pairIdx = pairIdx;
        fa.segs = segK;
        fa.factor = factor;
        fa.scratch = b->scratch.as<char>();
        fa.scratchOff = scratchOff;
        fa.ptOff = ptOff;
        fa.triOff = triOff;
        fa.edgeOff = edgeOff;
        fa.cutPts = cutPts;
        fa.cutKeys = cutKeys;
        fa.faceTris = faceTris;
        fa.faceEdges = faceEdges;
        fa.faceStatus = faceStatus;
        fa.faceNpts = faceNpts;
        fa.faceNtris = faceNtris;
        fa.faceNedges = faceNedges;
        fa.ptSrc = ptSrc;
        fa.robustEdges = (b->opts.robust & SB_ROBUST_EDGE_TOLERANCE) != 0;
        fa.scratchCap = (unsigned long long)totals[0];
        fa.frames = faceFrames;
        fa.filteredEarcut = fp64 ? 0 : 1;
        launch_faces(fa, s);
        SB_CUDA_CHECK(cudaGetLastError());
        // the re-triangulated triangles are numbered in the faces' processing order: on the second stream,
        // after the processing order and the re-triangulation, beside the weld
        SB_CUDA_CHECK(cudaEventRecord(b->sideDone, s)); // re-recorded: earlier waits hold their own records
        SB_CUDA_CHECK(cudaStreamWaitEvent(b->side, b->sideDone, 0));
        RankScanArgs rr;
        std::memset(&rr, 0, sizeof rr);
        rr.n = nFaces;
        rr.FA = FA;
        rr.count = 1;
        rr.faceByRank = faceByRank;
        rr.faceRank = faceRank;
        rr.vals[0] = faceNtris;
        rr.out[0] = retriRank;
        rr.tmp[0] = rankTmp[2];
        rr.tot[0] = rankTot + 4;
        rr.part = rankPart2;
        launch_rank_scan(rr, b->side);
        SB_CUDA_CHECK(cudaEventRecord(b->retriDone, b->side));
    }
    SB_CUDA_CHECK(cudaEventRecord(b->ev[3], s));

    // ---------------- statuses ----------------
    int firstFail[3] = {INT_MAX, INT_MAX, INT_MAX};
    // from the mailbox's constant area (three INT_MAX written when the boolean was created)
    SB_CUDA_CHECK(cudaMemcpyAsync(d_firstFail, b->mail + kMailRead, sizeof firstFail, cudaMemcpyHostToDevice, s));
    if (nFaces > 0)
        SB_COUNT(k_face_status)<<<blocks(nFaces, 256), 256, 0, s>>>(nFaces, faceSide, faceStatus, d_firstFail);

    // ---------------- global weld ----------------
    g.A = A;
    g.B = B;
    g.factor = factor;
    g.nFaces = nFaces;
    g.faceSide = faceSide;
    g.faceTri = faceTri;
    g.faceNpts = faceNpts;
    g.faceNtris = faceNtris;
    g.faceNedges = faceNedges;
    g.ptOff = ptOff;
    g.triOff = triOff;
    g.edgeOff = edgeOff;
    g.cutPts = cutPts;
    g.cutKeys = cutKeys;
    g.ptRef = ptRef;
    g.edgeRef = edgeRef;
    g.faceTris = faceTris;
    g.faceEdges = faceEdges;
    g.counters = d_counters;
    g.newBase = A.nv + B.nv;
    g.ptSrc = ptSrc;
    if (orderPending)
        SB_CUDA_CHECK(cudaStreamWaitEvent(s, b->orderDone, 0));
    launch_weld(g, s);
    SB_CUDA_CHECK(cub_run(b, [&](void *tmp, size_t &bytes) {
        return cub::DeviceScan::ExclusiveSum(tmp, bytes, g.isFirst, g.firstRank, (int)nSeq + 1, s);
    }));
    // the number of welded points is read with the arrangement's counts below (nothing before needs it)
    int nNew = 0;

    if (nFaces > 0)
        SB_CUDA_CHECK(cudaStreamWaitEvent(s, b->retriDone, 0));
    (void)retriRef;
    int cnts[4] = {0, 0, 0, 0}; // uncutA, uncutB, retriA, retri total
    {
        Readback rb(b);
        SB_CUDA_CHECK(rb.add(cnts, g.uncutRankA + nA, sizeof(int)));
        SB_CUDA_CHECK(rb.add(cnts + 1, g.uncutRankB + nB, sizeof(int)));
        if (nFaces > 0)
            SB_CUDA_CHECK(rb.add(cnts + 2, rankTot + 4, 2 * sizeof(int)));
        SB_CUDA_CHECK(rb.add(firstFail, d_firstFail, sizeof firstFail));
        SB_CUDA_CHECK(rb.add(&nNew, g.firstRank + nSeq, sizeof nNew));
        SB_CUDA_CHECK(rb.sync());
    }
    {
        // synchronised past the stream's wait for the leaf orders: their status is readable
        const sb_status r = rankResults();
        if (r != SB_OK)
            return r;
    }
    g.nNew = nNew;
    st.new_points = (uint64_t)nNew;
    const size_t nV = (size_t)A.nv + B.nv + nNew;
    g.useAdj = adjDup[0] == 0 && adjDup[1] == 0;
    g.uncutA = cnts[0];
    g.uncutB = cnts[1];
    g.retriRank = retriRank;
    const int nTri = cnts[0] + cnts[1] + cnts[3];
    g.nTri = nTri;
    b->nTri = nTri;

    // results block: vertices, arrangement triangles, labels, mesh tags, fetch outputs
    Carve cr;
    size_t o_V = cr.take<double>(3 * nV + 3), o_T = cr.take<uint32_t>(3 * (size_t)nTri + 3);
    size_t o_L = cr.take<int8_t>(nTri + 1), o_M = cr.take<int8_t>(nTri + 1), o_U = cr.take<int8_t>(nTri + 1);
    size_t o_F0 = cr.take<uint32_t>(3 * (size_t)nTri + 3), o_F1 = cr.take<uint32_t>(3 * (size_t)nTri + 3);
    size_t o_F2 = cr.take<uint32_t>(3 * (size_t)nTri + 3);
    size_t o_fl = cr.take<int>(3 * ((size_t)nTri + 1)), o_fr2 = cr.take<int>(3 * ((size_t)nTri + 1));
    size_t o_ou = cr.take<int>((size_t)cnts[0] + cnts[1] + 1), o_rf = cr.take<int>((size_t)cnts[3] + 1);
    SB_CUDA_CHECK(b->res.ensure(cr.off));
    char *rb = b->res.as<char>();
    g.newV = (double *)(rb + o_V);
    g.newT = (uint32_t *)(rb + o_T);
    g.label = (int8_t *)(rb + o_L);
    g.triMesh = (int8_t *)(rb + o_M);
    g.isUncut = (int8_t *)(rb + o_U);
    g.origUncut = (int *)(rb + o_ou);
    g.retriFace = (int *)(rb + o_rf);
    b->d_newV = g.newV;
    b->nNewV = nV;
    b->d_newT = g.newT;
    b->d_label = g.label;
    b->d_triMesh = g.triMesh;
    uint32_t *fetchOut[3] = {(uint32_t *)(rb + o_F0), (uint32_t *)(rb + o_F1), (uint32_t *)(rb + o_F2)};
    int *fFlag = (int *)(rb + o_fl), *fRank = (int *)(rb + o_fr2);
    if (A.nv > 0)
        SB_CUDA_CHECK(cudaMemcpyAsync(g.newV, A.v, sizeof(double) * 3 * A.nv, cudaMemcpyDeviceToDevice, s));
    if (B.nv > 0)
        SB_CUDA_CHECK(
            cudaMemcpyAsync(g.newV + 3 * (size_t)A.nv, B.v, sizeof(double) * 3 * B.nv, cudaMemcpyDeviceToDevice, s));
    launch_weld_number(g, (int)nSeq, s);
    if (b->opts.stage_results && nV > 0) {
        // the result vertices are final: copied to the host on the copy stream beside the rest
        if (!b->stage) {
            SB_CUDA_CHECK(cudaStreamCreateWithFlags(&b->stage, cudaStreamNonBlocking));
            SB_CUDA_CHECK(cudaEventCreateWithFlags(&b->stageEv, cudaEventDisableTiming));
        }
        void *hv = nullptr;
        if (sb_host_alloc(sizeof(double) * 3 * nV, &hv) == SB_OK && hv) {
            b->staged[SB_STAGED_VERTICES] = sb_boolean::Staged{hv, nV};
            SB_CUDA_CHECK(cudaEventRecord(b->stageEv, s));
            SB_CUDA_CHECK(cudaStreamWaitEvent(b->stage, b->stageEv, 0));
            b->staging = true;
            SB_CUDA_CHECK(cudaMemcpyAsync(hv, g.newV, sizeof(double) * 3 * nV, cudaMemcpyDeviceToHost, b->stage));
        }
    }
    if (nTri > 0)
        SB_COUNT(k_tri_mesh)<<<blocks(nTri, 256), 256, 0, s>>>(nTri, cnts[0], cnts[1], cnts[2], g.triMesh, g.isUncut);
    launch_arrangement(g, s);
    SB_CUDA_CHECK(cudaGetLastError());
    SB_CUDA_CHECK(cudaEventRecord(b->ev[4], s));

    // ---------------- cut loops, groups, sides ----------------
    const uint32_t edgeCapH = pow2_at_least(2 * (size_t)totals[3] + 2);
    // per-mesh half-edge tables: every arrangement triangle's, or through the input adjacency only the
    // re-triangulated triangles'
    const uint32_t heCap = pow2_at_least(2 * 3 * (size_t)(g.useAdj ? cnts[3] : nTri) + 2);
    Carve cg2;
    size_t o_ek = cg2.take<uint64_t>(edgeCapH), o_ev = cg2.take<int>(edgeCapH), o_dg = cg2.take<int>(nNew + 1);
    size_t o_esl = cg2.take<int>(edgeCapH), o_esh = cg2.take<int>(edgeCapH), o_fo = cg2.take<int>(nNew + 1);
    size_t o_nb = cg2.take<int>(2 * (size_t)nNew + 2), o_nbs = cg2.take<int>(2 * (size_t)nNew + 2);
    const size_t nQueryCap = (size_t)nTri + 4 * (size_t)nNew + 1;
    size_t o_hkA = cg2.take<uint64_t>(heCap), o_hvA = cg2.take<int>(heCap);
    size_t o_hkB = cg2.take<uint64_t>(heCap), o_hvB = cg2.take<int>(heCap);
    size_t o_par = cg2.take<int>(nTri + 1), o_sf = cg2.take<int>(nTri + 1), o_smn = cg2.take<int>(nTri + 1);
    size_t o_rmn = cg2.take<int>(nTri + 1), o_ror = cg2.take<int>(nTri + 1), o_rep = cg2.take<int>(nQueryCap);
    size_t o_ins = cg2.take<int>(nQueryCap);

    SB_CUDA_CHECK(b->groups.ensure(cg2.off));
    char *gb = b->groups.as<char>();
    g.edgeKeys = (uint64_t *)(gb + o_ek);
    g.edgeVals = (int *)(gb + o_ev);
    g.edgeMask = edgeCapH - 1;
    g.degree = (int *)(gb + o_dg);
    g.edgeSlotLo = (int *)(gb + o_esl);
    g.edgeSlotHi = (int *)(gb + o_esh);
    g.firstOcc = (int *)(gb + o_fo);
    g.nbr = (int *)(gb + o_nb);
    g.nbrSlot = (int *)(gb + o_nbs);
    g.heKeysA = (uint64_t *)(gb + o_hkA);
    g.heValsA = (int *)(gb + o_hvA);
    g.heKeysB = (uint64_t *)(gb + o_hkB);
    g.heValsB = (int *)(gb + o_hvB);
    g.heMask = heCap - 1;
    g.parent = (int *)(gb + o_par);
    g.seedFlag = (int *)(gb + o_sf);
    g.seedMin = (int *)(gb + o_smn);
    g.remMin = (int *)(gb + o_rmn);
    g.repOfRoot = (int *)(gb + o_ror);
    g.qTri = (int *)(gb + o_rep);
    g.insideCount = (int *)(gb + o_ins);

    {
        // the loop tables and every grouping table, in one launch before the loops
        Fills fl(s);
        fl.u64(g.edgeKeys, edgeCapH, kEmpty64);
        fl.i32(g.edgeVals, edgeCapH, INT_MAX);
        fl.i32(g.degree, (size_t)nNew + 1, 0);
        fl.i32(g.edgeSlotLo, edgeCapH, INT_MAX);
        fl.i32(g.edgeSlotHi, edgeCapH, INT_MAX);
        fl.i32(g.firstOcc, (size_t)nNew + 1, INT_MAX);
        fl.i32(g.nbr, 2 * (size_t)nNew + 2, -1);
        fl.i32(g.nbrSlot, 2 * (size_t)nNew + 2, -1);
        fl.u64(g.heKeysA, heCap, kEmpty64);
        fl.u64(g.heKeysB, heCap, kEmpty64);
        fl.i32(g.heValsA, heCap, INT_MAX);
        fl.i32(g.heValsB, heCap, INT_MAX);
        if (nTri > 0) {
            fl.iota(g.parent, nTri);
            fl.i32(g.seedMin, nTri, INT_MAX);
            fl.i32(g.remMin, nTri, INT_MAX);
            fl.i32(g.repOfRoot, nTri, -1);
            fl.i32(g.insideCount, nQueryCap, 0);
        }
        fl.launch();
    }
    launch_loops(g, s);
    // the loops in the reference's order, the group seeds and each group's first triangle
    const size_t nNewS = (size_t)std::max(nNew, 1), nTriS = (size_t)std::max(nTri, 1);
    const int slotDomain = 4 * (int)K; // first-mesh faces hold 2 K directed cut-edge slots, two sequence slots each
    Carve cl;
    const size_t o_st = cl.take<int>(4 * nNewS), o_el = cl.take<int>(nNewS), o_fq = cl.take<int>(nTriS);
    const size_t o_g0 = cl.take<int>(4 * nNewS), o_gq = cl.take<int>(4 * nNewS), o_inf = cl.take<int>(4);
    const size_t o_lsc = cl.take<int>(loop_order_scratch_ints(slotDomain, nNew));
    const size_t o_irk = cl.take<int>(nNewS), o_lkeys = cl.take<uint32_t>(nNewS), o_vis = cl.take<int2>(2 * nNewS);
    const size_t o_ho = cl.take<int>(nNewS), o_lhs = cl.take<int>(hash_scratch_ints(nNew));
    const size_t o_eb = cl.take<int>(nNewS), o_en = cl.take<int>(nNewS);
    const size_t o_rsn = cl.take<int>(nTriS), o_rsx = cl.take<int>(nTriS), o_bg = cl.take<int>(nTriS);
    const size_t o_be = cl.take<int>(nTriS), o_f0 = cl.take<int>(nTriS), o_f1 = cl.take<int>(nTriS);
    const size_t o_tg = cl.take<int>(3 * nTriS), o_ffl = cl.take<int>(std::max(3 * nTriS, 4 * nNewS) + 1);
    const size_t o_any = cl.take<int>(1);
    SB_CUDA_CHECK(b->flood.ensure(cl.off));
    char *lb = b->flood.as<char>();
    LoopOrderArgs lo;
    lo.nNew = nNew;
    lo.nTri = nTri;
    lo.newBase = (uint32_t)g.newBase;
    lo.slotDomain = slotDomain;
    lo.degree = g.degree;
    lo.nbr = g.nbr;
    lo.nbrSlot = g.nbrSlot;
    lo.firstOcc = g.firstOcc;
    lo.loopBad = d_counters + kCntLoopVerts + 1;
    lo.loopErr = d_counters + kCntSideErrors;
    lo.heKeysA = g.heKeysA;
    lo.heKeysB = g.heKeysB;
    lo.heValsA = g.heValsA;
    lo.heValsB = g.heValsB;
    lo.heMask = g.heMask;
    lo.seedTri = (int *)(lb + o_st);
    lo.entryLoop = (int *)(lb + o_el);
    lo.firstQ = (int *)(lb + o_fq);
    lo.group0 = (int *)(lb + o_g0);
    lo.gQuery = (int *)(lb + o_gq);
    lo.qTri = g.qTri;
    lo.qCount = d_counters + kCntReps;
    lo.info = (int *)(lb + o_inf);
    lo.scratch = (int *)(lb + o_lsc);
    lo.insRank = (int *)(lb + o_irk);
    lo.insKeys = (uint32_t *)(lb + o_lkeys);
    lo.vis = (int2 *)(lb + o_vis);
    lo.hashOut = (int *)(lb + o_ho);
    lo.hs = hash_scratch_at((int *)(lb + o_lhs), nNew);
    lo.entryBase = (int *)(lb + o_eb);
    lo.entryNext = (int *)(lb + o_en);
    lo.smemInts = 0;
    lo.stamps = reinterpret_cast<unsigned long long *>(b->small.as<char>() + 1024); // [8] after the counters
    FloodArgs fd;
    fd.nTri = nTri;
    fd.nNew = nNew;
    fd.root = g.parent;
    fd.seedMin = g.seedMin;
    fd.seedTri = lo.seedTri;
    fd.firstQ = lo.firstQ;
    fd.entryLoop = lo.entryLoop;
    fd.gQuery = lo.gQuery;
    fd.info = lo.info;
    fd.insideCount = g.insideCount;
    fd.regionQuery = g.repOfRoot;
    fd.rsMin = (int *)(lb + o_rsn);
    fd.rsMax = (int *)(lb + o_rsx);
    fd.bfsGroup = (int *)(lb + o_bg);
    fd.best = (int *)(lb + o_be);
    fd.front0 = (int *)(lb + o_f0);
    fd.front1 = (int *)(lb + o_f1);
    fd.tgt = (int *)(lb + o_tg);
    fd.flag = (int *)(lb + o_ffl);
    fd.anyMixed = (int *)(lb + o_any);
    fd.errors = d_counters + kCntSideErrors;
    {
        Fills fl(s);
        fl.i32(lo.firstQ, nTriS, INT_MAX);
        fl.i32(lo.info, 4, 0);
        fl.i32(fd.rsMin, nTriS, 2);
        fl.i32(fd.rsMax, nTriS, -1);
        fl.i32(fd.bfsGroup, nTriS, -1);
        fl.i32(fd.best, nTriS, INT_MAX);
        fl.i32(fd.anyMixed, 1, 0);
        fl.launch();
    }
    // The loop order needs the loop tables only: it runs on the second stream beside the half-edge tables and
    // the union-find regions; the seeds after it wait for the half-edge tables as well.
    SB_CUDA_CHECK(cudaEventRecord(b->sideDone, s));
    SB_CUDA_CHECK(cudaStreamWaitEvent(b->side, b->sideDone, 0));
    launch_loop_order(lo, b->side);
    launch_halfedges(g, s);
    SB_CUDA_CHECK(cudaEventRecord(b->sideDone, s)); // re-recorded: the wait above already holds the first one
    SB_CUDA_CHECK(cudaStreamWaitEvent(b->side, b->sideDone, 0));
    launch_seed_entries(lo, b->side);
    SB_CUDA_CHECK(cudaEventRecord(b->orderDone, b->side));
    launch_groups(g, s);
    SB_CUDA_CHECK(cudaStreamWaitEvent(s, b->orderDone, 0));
    launch_side_queries(g, lo, s);
    SB_CUDA_CHECK(cudaGetLastError());
    SB_CUDA_CHECK(cudaEventRecord(b->ev[5], s));
    unsigned int counters[kCntCount];
    {
        sb_status r = read_back(b, counters, d_counters, sizeof counters);
        if (r != SB_OK)
            return r;
    }
    const unsigned int nQueries = counters[kCntReps];
    SB_CUDA_CHECK(b->sides.ensure(side_layout(g, 3 * (int)nQueries, nullptr)));
    side_layout(g, 3 * (int)nQueries, b->sides.as<char>());
    launch_sides(g, nQueries, fp64, s);
    launch_flood_labels(g, fd, s);
    SB_CUDA_CHECK(cudaGetLastError());
    SB_CUDA_CHECK(cudaEventRecord(b->ev[6], s));

    // ---------------- status ----------------
    sb_status status = SB_OK;
    if (firstFail[2] != INT_MAX)
        status = SB_ERR_CAPACITY;
    else if (firstFail[0] != INT_MAX || firstFail[1] != INT_MAX) {
        int f = firstFail[0] != INT_MAX ? firstFail[0] : firstFail[1];
        int code = 0;
        {
            const sb_status r = read_back(b, &code, faceStatus + f, sizeof code);
            if (r != SB_OK)
                return r;
        }
        status = code == 1 ? SB_FAIL_ATTACH : SB_FAIL_LINK;
    } else if (counters[kCntLoopVerts + 1] != 0)
        status = SB_FAIL_LOOP;

    // ---------------- fetch ----------------
    if (status == SB_OK && nTri > 0) {
        // the three fetch compactions: one flag pass, one scan over the three runs, one write pass; their
        // sizes are read with the final statistics
        launch_fetch_flags(g, fFlag, s);
        SB_CUDA_CHECK(cub_run(b, [&](void *tmp, size_t &bytes) {
            return cub::DeviceScan::ExclusiveSum(tmp, bytes, fFlag, fRank, 3 * (nTri + 1), s);
        }));
        launch_fetch_write(g, fFlag, fRank, fetchOut, s);
    }
    SB_CUDA_CHECK(cudaEventRecord(b->ev[7], s));
    unsigned long long dstats[8];
    int runEnd[3] = {0, 0, 0}; // scan values where the three fetch runs end
    unsigned int orderFallbacks = 0;
    int loopInfo[2] = {0, 0};
    {
        Readback rb(b);
        SB_CUDA_CHECK(rb.add(dstats, d_stats, sizeof dstats));
        SB_CUDA_CHECK(rb.add(counters, d_counters, sizeof counters));
        SB_CUDA_CHECK(rb.add(&orderFallbacks, d_counters + kCntCount, sizeof orderFallbacks));
        SB_CUDA_CHECK(rb.add(loopInfo, lo.info, sizeof loopInfo));
        if (status == SB_OK && nTri > 0)
            for (int op = 0; op < 3; ++op)
                SB_CUDA_CHECK(rb.add(runEnd + op, fRank + op * ((size_t)nTri + 1) + nTri, sizeof(int)));
        SB_CUDA_CHECK(rb.sync());
    }
    if (status == SB_OK && nTri > 0)
        for (int op = 0; op < 3; ++op) {
            b->d_fetch[op] = fetchOut[op];
            b->nFetch[op] = (size_t)(runEnd[op] - (op > 0 ? runEnd[op - 1] : 0));
        }
    SB_CUDA_CHECK(cudaGetLastError());
    {
        const sb_status r = rankResults();
        if (r != SB_OK)
            return r;
    }
    st.box_tests = dstats[0];
    st.box_fallbacks = dstats[1];
    st.sign_tests = dstats[2];
    st.sign_fallbacks = dstats[3];
    if (dstats[4] != 0 || counters[kCntSideErrors] != 0)
        status = SB_ERR_CAPACITY;
    st.result_vertices = nV;
    st.result_triangles = (uint64_t)nTri;
    st.regions_first = counters[kCntRegionsA];
    st.regions_second = counters[kCntRegionsA + 1];
    st.loop_vertices = counters[kCntLoopVerts];
    st.loop_bad_degree = counters[kCntLoopVerts + 1];
    st.duplicate_halfedges = counters[kCntDupHalfedge];
    st.loops = (uint32_t)loopInfo[1];
    st.order_fallbacks = orderFallbacks;
    for (int k = 0; k < 7; ++k) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, b->ev[k], b->ev[k + 1]);
        st.stage_ms[k] = ms;
    }
    if (b->opts.stage_results && status == SB_OK) {
        // the three fetch results, sized now, in one more round trip; the vertices' copy ended long ago
        for (int op = 0; op < 3; ++op) {
            const size_t n = b->nFetch[op];
            void *h = nullptr;
            if (n && sb_host_alloc(sizeof(uint32_t) * 3 * n, &h) == SB_OK && h) {
                b->staged[op] = sb_boolean::Staged{h, n};
                SB_CUDA_CHECK(cudaMemcpyAsync(h, b->d_fetch[op], sizeof(uint32_t) * 3 * n, cudaMemcpyDeviceToHost, s));
            }
        }
        SB_CUDA_CHECK(cudaStreamSynchronize(s));
    }
    SB_CUDA_CHECK(staged_wait(b));
    b->status = status;
    b->combined = true;
    return status;
}

} // namespace

// ---------------------------------------------------------------------------------------------------
// exported functions
// ---------------------------------------------------------------------------------------------------
extern "C" {

void sb_default_options(sb_options *o)
{
    if (!o)
        return;
    o->weld_factor = 100000;
    o->precision = SB_PRECISION_FILTERED;
    o->order = SB_ORDER_REFERENCE;
    o->stream = nullptr;
    o->robust = 0;
    o->stage_results = 0;
}

const char *sb_status_string(sb_status s)
{
    switch (s) {
    case SB_OK: return "ok";
    case SB_FAIL_ATTACH: return "attach point to triangle edge failed";
    case SB_FAIL_LINK: return "polygon ring link failed";
    case SB_FAIL_LOOP: return "cut edges do not form closed loops";
    case SB_ERR_INVALID: return "invalid argument";
    case SB_ERR_CUDA: return "CUDA error";
    case SB_ERR_CAPACITY: return "capacity bound exceeded";
    case SB_ERR_NOT_COMBINED: return "not combined";
    }
    return "unknown";
}

const char *sb_last_error(void) { return g_last_error.c_str(); }

uint64_t sb_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

void sb_kernel_timing(int enable)
{
    std::lock_guard<std::mutex> lk(g_kt_mutex);
    g_kt_used = 0;
    g_kt_on.store(enable != 0);
}

void sb_kernel_timing_select(const char *names)
{
    std::lock_guard<std::mutex> lk(g_kt_mutex);
    g_kt_only = names && *names ? "," + std::string(names) + "," : std::string();
}

int sb_kernel_timing_read(const char *name, double *total_ms, uint64_t *launches)
{
    std::lock_guard<std::mutex> lk(g_kt_mutex);
    double tot = 0.0;
    uint64_t n = 0;
    for (size_t i = 0; i < g_kt_used; ++i) {
        if (g_kt_recs[i].name != name)
            continue;
        if (cudaEventSynchronize(g_kt_recs[i].b) != cudaSuccess)
            return -1;
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, g_kt_recs[i].a, g_kt_recs[i].b) != cudaSuccess)
            return -1;
        tot += ms;
        ++n;
    }
    if (total_ms)
        *total_ms = tot;
    if (launches)
        *launches = n;
    return 0;
}

int sb_kernel_timing_names(char *buf, size_t cap)
{
    std::lock_guard<std::mutex> lk(g_kt_mutex);
    std::string all;
    for (size_t i = 0; i < g_kt_used; ++i) {
        const std::string &n = g_kt_recs[i].name;
        if (("," + all + ",").find("," + n + ",") == std::string::npos)
            all += (all.empty() ? "" : ",") + n;
    }
    if (buf && cap) {
        std::strncpy(buf, all.c_str(), cap - 1);
        buf[cap - 1] = 0;
    }
    return (int)all.size();
}

static sb_status mesh_alloc(size_t nv, size_t nt, sb_mesh **out)
{
    if (!out || nv > 0x7FFFFFFFu || nt > 0x2AAAAAAAu) {
        set_last_error("mesh too large or null output");
        return SB_ERR_INVALID;
    }
    auto *m = new sb_mesh;
    m->d.nv = (int)nv;
    m->d.nt = (int)nt;
    cudaError_t e = m->buf.ensure(mesh_bytes((int)nv, (int)nt));
    if (e != cudaSuccess) {
        delete m;
        return cuda_fail(e, "cudaMalloc(mesh)", __FILE__, __LINE__);
    }
    Carve c;
    size_t o_v = c.take<double>(nv * 3);
    size_t o_t = c.take<uint32_t>(nt * 3);
    m->d.v = reinterpret_cast<double *>(m->buf.as<char>() + o_v);
    m->d.t = reinterpret_cast<uint32_t *>(m->buf.as<char>() + o_t);
    *out = m;
    return SB_OK;
}

static sb_status mesh_validate(sb_mesh *m, cudaStream_t s)
{
    if (m->d.nt == 0)
        return SB_OK;
    unsigned int *d_bad = reinterpret_cast<unsigned int *>(m->buf.as<char>() + mesh_layout_bytes(m->d.nv, m->d.nt));
    SB_CUDA_CHECK(cudaMemsetAsync(d_bad, 0, sizeof(unsigned int), s));
    SB_COUNT(k_validate_tris)<<<blocks(3 * (size_t)m->d.nt, 256), 256, 0, s>>>(m->d.nt, m->d.nv, m->d.t, d_bad);
    // the mesh's pinned slot: ints [0, 12) hold the leaf-order status, the last one this flag
    if (!m->rankCheck && !(m->rankCheck = pinned_slot_acquire())) {
        set_last_error("no pinned host memory for the mesh");
        return SB_ERR_CUDA;
    }
    SB_CUDA_CHECK(cudaMemcpyAsync(m->rankCheck + 15, d_bad, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
    SB_CUDA_CHECK(cudaStreamSynchronize(s));
    if (m->rankCheck[15]) {
        set_last_error("triangle index out of range");
        return SB_ERR_INVALID;
    }
    return SB_OK;
}

sb_status sb_mesh_create(const double *xyz, size_t nv, const uint32_t *tris, size_t nt, sb_mesh **out)
{
    return guarded([&]() -> sb_status {
        if ((nv && !xyz) || (nt && !tris))
            return SB_ERR_INVALID;
        sb_status r = mesh_alloc(nv, nt, out);
        if (r != SB_OK)
            return r;
        sb_mesh *m = *out;
        // both uploads and the index check in stream order, one host round trip (the check's read-back waits
        // for the copies, so the caller's arrays are free again when this returns)
        if (nv)
            SB_CUDA_CHECK(cudaMemcpyAsync(m->d.v, xyz, sizeof(double) * 3 * nv, cudaMemcpyHostToDevice, nullptr));
        if (nt)
            SB_CUDA_CHECK(cudaMemcpyAsync(m->d.t, tris, sizeof(uint32_t) * 3 * nt, cudaMemcpyHostToDevice, nullptr));
        r = mesh_validate(m, nullptr);
        if (r == SB_OK && nt == 0 && nv)
            SB_CUDA_CHECK(cudaStreamSynchronize(nullptr)); // no check ran: wait for the vertex copy
        if (r != SB_OK) {
            sb_mesh_destroy(m);
            *out = nullptr;
        }
        return r;
    });
}

sb_status sb_mesh_create_device(const double *d_xyz, size_t nv, const uint32_t *d_tris, size_t nt,
                                const sb_options *opts, sb_mesh **out)
{
    return guarded([&]() -> sb_status {
        if ((nv && !d_xyz) || (nt && !d_tris))
            return SB_ERR_INVALID;
        sb_status r = mesh_alloc(nv, nt, out);
        if (r != SB_OK)
            return r;
        sb_mesh *m = *out;
        cudaStream_t s = opts ? (cudaStream_t)opts->stream : nullptr;
        m->stream = s;
        if (nv)
            SB_CUDA_CHECK(cudaMemcpyAsync(m->d.v, d_xyz, sizeof(double) * 3 * nv, cudaMemcpyDeviceToDevice, s));
        if (nt)
            SB_CUDA_CHECK(cudaMemcpyAsync(m->d.t, d_tris, sizeof(uint32_t) * 3 * nt, cudaMemcpyDeviceToDevice, s));
        r = mesh_validate(m, s);
        if (r != SB_OK) {
            sb_mesh_destroy(m);
            *out = nullptr;
        }
        return r;
    });
}

sb_status sb_mesh_update_vertices_device(sb_mesh *m, const double *d_xyz, const sb_options *opts)
{
    if (!m || (m->d.nv && !d_xyz))
        return SB_ERR_INVALID;
    cudaStream_t s = opts ? (cudaStream_t)opts->stream : nullptr;
    {
        const sb_status r = mesh_order_after(m, s); // a pending build may still read the vertices
        if (r != SB_OK)
            return r;
    }
    if (m->d.nv)
        SB_CUDA_CHECK(cudaMemcpyAsync(m->d.v, d_xyz, sizeof(double) * 3 * m->d.nv, cudaMemcpyDeviceToDevice, s));
    m->prepared = false;
    return SB_OK;
}

sb_status sb_mesh_prepare(sb_mesh *m, const sb_options *opts)
{
    if (!m)
        return SB_ERR_INVALID;
    return guarded([&]() -> sb_status {
        sb_options o;
        sb_default_options(&o);
        if (opts)
            o = *opts;
        // issued without waiting: sb_combine orders itself after the build and reports its status
        cudaStream_t s = (cudaStream_t)o.stream;
        if (!s) {
            // no stream given: the build runs on the mesh's own stream, after everything queued so far on the
            // legacy default stream, so that two meshes prepared one after the other build concurrently
            if (!m->own) {
                SB_CUDA_CHECK(cudaStreamCreateWithFlags(&m->own, cudaStreamNonBlocking));
                SB_CUDA_CHECK(cudaEventCreateWithFlags(&m->ownFork, cudaEventDisableTiming));
            }
            SB_CUDA_CHECK(cudaEventRecord(m->ownFork, nullptr));
            SB_CUDA_CHECK(cudaStreamWaitEvent(m->own, m->ownFork, 0));
            s = m->own;
        }
        return prepare_mesh(m, o.order, s, false);
    });
}

void sb_mesh_destroy(sb_mesh *m)
{
    if (!m)
        return;
    m->buf.release();
    m->tmp.release();
    m->rankTmp.release();
    if (m->rankPending && m->aux)
        cudaStreamSynchronize(m->aux);
    pinned_slot_release(m->rankCheck);
    if (m->aux)
        cudaStreamDestroy(m->aux);
    if (m->own) {
        cudaStreamSynchronize(m->own);
        cudaStreamDestroy(m->own);
        cudaEventDestroy(m->ownFork);
    }
    if (m->auxFork)
        cudaEventDestroy(m->auxFork);
    if (m->auxJoin)
        cudaEventDestroy(m->auxJoin);
    if (m->readyEv)
        cudaEventDestroy(m->readyEv);
    delete m;
}

sb_status sb_boolean_create(const sb_mesh *first, const sb_mesh *second, const sb_options *opts, sb_boolean **out)
{
    if (!first || !second || !out)
        return SB_ERR_INVALID;
    return guarded([&]() -> sb_status {
        auto *b = new sb_boolean;
        b->first = first;
        b->second = second;
        sb_default_options(&b->opts);
        if (opts)
            b->opts = *opts;
        if (b->opts.weld_factor <= 0) {
            delete b;
            return SB_ERR_INVALID;
        }
        b->s = (cudaStream_t)b->opts.stream;
        std::memset(&b->stats, 0, sizeof b->stats);
        b->mail = pinned_mail_acquire();
        if (!b->mail) {
            delete b;
            set_last_error("no pinned host memory for the boolean's mailbox");
            return SB_ERR_CUDA;
        }
        const int big[3] = {INT_MAX, INT_MAX, INT_MAX};
        std::memcpy(b->mail + kMailRead, big, sizeof big);
        *out = b;
        return SB_OK;
    });
}

static bool is_combine_failure(sb_status r)
{
    return r == SB_FAIL_ATTACH || r == SB_FAIL_LINK || r == SB_FAIL_LOOP;
}

// Largest absolute vertex coordinate of a prepared mesh: its hierarchy's root box (FP64 unions of the
// triangle boxes, which hold the vertices' exact minima and maxima). Synchronises the stream.
static sb_status mesh_max_abs(const sb_mesh *m, cudaStream_t s, double *out)
{
    const MeshDev &d = m->d;
    *out = 0.0;
    if (d.nt <= 0)
        return SB_OK;
    double box[6];
    const double *src = d.nt == 1 ? d.box64 : d.nbox64; // node 0 is the root
    SB_CUDA_CHECK(cudaMemcpyAsync(box, src, sizeof box, cudaMemcpyDeviceToHost, s));
    SB_CUDA_CHECK(cudaStreamSynchronize(s));
    for (double x : box)
        *out = std::max(*out, std::fabs(x));
    return SB_OK;
}

sb_status sb_combine(sb_boolean *b, sb_stats *stats)
{
    if (!b)
        return SB_ERR_INVALID;
    return guarded([&]() -> sb_status {
        sb_mesh *ma = const_cast<sb_mesh *>(b->first), *mb = const_cast<sb_mesh *>(b->second);
        if (!ma->prepared && !mb->prepared && ma != mb) {
            // both meshes need preparing: the second one on a side stream, so the two latency-bound builds
            // overlap on the device (issuing never blocks the host); the main stream then waits for the side
            if (!b->side) {
                SB_CUDA_CHECK(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking));
                SB_CUDA_CHECK(cudaEventCreateWithFlags(&b->sideDone, cudaEventDisableTiming));
            }
            SB_CUDA_CHECK(cudaEventRecord(b->sideDone, b->s));
            SB_CUDA_CHECK(cudaStreamWaitEvent(b->side, b->sideDone, 0));
            const sb_status r = prepare_meshes(ma, b->s, mb, b->side, b->opts.order);
            if (r != SB_OK)
                return r;
            SB_CUDA_CHECK(cudaEventRecord(b->sideDone, b->side));
            SB_CUDA_CHECK(cudaStreamWaitEvent(b->s, b->sideDone, 0));
        }
        for (sb_mesh *m : {ma, mb})
            if (!m->prepared) {
                sb_status r = prepare_mesh(m, b->opts.order, b->s, false);
                if (r != SB_OK)
                    return r;
            }
        sb_status r = combine_impl(b);
        uint32_t attempts = 1;
        const int64_t factor0 = b->opts.weld_factor;
        if (is_combine_failure(r) && (b->opts.robust & SB_ROBUST_WELD_RETRY)) {
            // the finer quanta: x10 while the factor stays <= 1e12 and coarser than FP64's resolution
            double absA = 0.0, absB = 0.0;
            sb_status e = mesh_max_abs(ma, b->s, &absA);
            if (e == SB_OK)
                e = mesh_max_abs(mb, b->s, &absB);
            if (e != SB_OK)
                return e;
            const double maxAbs = std::max(absA, absB);
            while (is_combine_failure(r) && b->opts.weld_factor <= 100000000000LL &&
                   maxAbs * (double)(b->opts.weld_factor * 10) < 4503599627370496.0) {
                b->opts.weld_factor *= 10;
                r = combine_impl(b);
                ++attempts;
            }
        }
        b->stats.attempts = attempts;
        b->stats.robust = b->opts.robust;
        b->stats.weld_factor_used = b->opts.weld_factor;
        b->opts.weld_factor = factor0; // the next combine starts from the caller's factor again
        if (stats)
            *stats = b->stats;
        return r;
    });
}

static sb_status check_fetchable(sb_boolean *b)
{
    if (!b)
        return SB_ERR_INVALID;
    if (!b->combined)
        return SB_ERR_NOT_COMBINED;
    return SB_OK;
}

sb_status sb_fetch(sb_boolean *b, sb_op op, uint32_t *tris, size_t cap, size_t *count)
{
    sb_status r = check_fetchable(b);
    if (r != SB_OK)
        return r;
    if (op < SB_UNION || op > SB_INTERSECT || !count)
        return SB_ERR_INVALID;
    size_t n = b->status == SB_OK ? b->nFetch[op] : 0;
    *count = n;
    if (!tris)
        return SB_OK;
    if (cap < n)
        return SB_ERR_INVALID;
    if (n)
        SB_CUDA_CHECK(cudaMemcpy(tris, b->d_fetch[op], sizeof(uint32_t) * 3 * n, cudaMemcpyDeviceToHost));
    return SB_OK;
}

sb_status sb_take_staged(sb_boolean *b, int32_t what, void **host, size_t *count)
{
    sb_status r = check_fetchable(b);
    if (r != SB_OK)
        return r;
    if (what < SB_UNION || what > SB_STAGED_VERTICES || !host || !count)
        return SB_ERR_INVALID;
    *count = what == SB_STAGED_VERTICES ? b->nNewV : (b->status == SB_OK ? b->nFetch[what] : 0);
    *host = b->staged[what].ptr;
    b->staged[what] = sb_boolean::Staged{};
    return SB_OK;
}

sb_status sb_fetch_device(sb_boolean *b, sb_op op, const uint32_t **d_tris, size_t *count)
{
    sb_status r = check_fetchable(b);
    if (r != SB_OK)
        return r;
    if (op < SB_UNION || op > SB_INTERSECT || !count || !d_tris)
        return SB_ERR_INVALID;
    *count = b->status == SB_OK ? b->nFetch[op] : 0;
    *d_tris = b->d_fetch[op];
    return SB_OK;
}

sb_status sb_result_vertices(sb_boolean *b, double *xyz, size_t cap, size_t *count)
{
    sb_status r = check_fetchable(b);
    if (r != SB_OK)
        return r;
    if (!count)
        return SB_ERR_INVALID;
    *count = b->nNewV;
    if (!xyz)
        return SB_OK;
    if (cap < b->nNewV)
        return SB_ERR_INVALID;
    if (b->nNewV)
        SB_CUDA_CHECK(cudaMemcpy(xyz, b->d_newV, sizeof(double) * 3 * b->nNewV, cudaMemcpyDeviceToHost));
    return SB_OK;
}

sb_status sb_result_vertices_device(sb_boolean *b, const double **d_xyz, size_t *count)
{
    sb_status r = check_fetchable(b);
    if (r != SB_OK)
        return r;
    if (!count || !d_xyz)
        return SB_ERR_INVALID;
    *count = b->nNewV;
    *d_xyz = b->d_newV;
    return SB_OK;
}

sb_status sb_debug_dump(sb_boolean *b, const char *name, void *out, size_t cap_bytes, size_t *bytes)
{
    sb_status r = check_fetchable(b);
    if (r != SB_OK)
        return r;
    if (!name || !bytes)
        return SB_ERR_INVALID;
    std::string n(name);
    const void *src = nullptr;
    size_t sz = 0;
    DevBuf tmp;
    if (n == "candidates") {
        sz = sizeof(uint32_t) * 2 * (size_t)b->C;
        if (out && sz) {
            SB_CUDA_CHECK(tmp.ensure(sz));
            SB_COUNT(k_cand_pairs)<<<blocks(b->C, 256), 256, 0, b->s>>>(b->C, b->d_cand, b->second->d.nt, tmp.as<uint32_t>());
            SB_CUDA_CHECK(cudaStreamSynchronize(b->s));
            src = tmp.ptr;
        }
    } else if (n == "intersection_pairs") {
        sz = sizeof(uint32_t) * 2 * (size_t)b->K;
        src = b->d_pairAB;
    } else if (n == "intersection_segments") {
        sz = sizeof(double) * 6 * (size_t)b->K;
        src = b->d_segK;
    } else if (n == "arrangement") {
        sz = sizeof(uint32_t) * 3 * (size_t)b->nTri;
        src = b->d_newT;
    } else if (n == "labels") {
        sz = (size_t)b->nTri;
        src = b->d_label;
    } else if (n == "tri_mesh") {
        sz = (size_t)b->nTri;
        src = b->d_triMesh;
    } else if (n == "new_sources") {
        // per appended vertex: 2 x (its intersecting pair) + (which end of that pair's segment)
        sz = sizeof(int) * (b->nNewV - (size_t)b->newBase);
        src = b->d_newSrc;
    } else if (n == "loop_order_ns") {
        // device time stamps (ns) at the phase boundaries of the loop-order kernel of the last combine
        sz = sizeof(unsigned long long) * 8;
        src = b->small.as<char>() + 1024;
    } else if (n == "leaf_order_ns_first" || n == "leaf_order_ns_second") {
        // device time stamps (ns) of the leaf-order build's large-node levels: start, classified, split
        const MeshDev &M = n == "leaf_order_ns_first" ? b->first->d : b->second->d;
        sz = M.levelStamps ? sizeof(unsigned long long) * 96 : 0;
        src = M.levelStamps;
    } else if (n == "rank_first" || n == "rank_second") {
        const MeshDev &M = n == "rank_first" ? b->first->d : b->second->d;
        sz = M.rankValid ? sizeof(int) * (size_t)M.nt : 0;
        src = M.rank;
    } else {
        return SB_ERR_INVALID;
    }
    *bytes = sz;
    if (!out || !sz) {
        tmp.release();
        return SB_OK;
    }
    if (cap_bytes < sz) {
        tmp.release();
        return SB_ERR_INVALID;
    }
    cudaError_t e = cudaMemcpy(out, src, sz, cudaMemcpyDeviceToHost);
    tmp.release();
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaMemcpy(dump)", __FILE__, __LINE__);
    return SB_OK;
}

void sb_boolean_destroy(sb_boolean *b)
{
    if (!b)
        return;
    for (DevBuf *d : {&b->cand, &b->isect, &b->faces, &b->scratch, &b->cut, &b->weld, &b->arr, &b->groups, &b->res,
                      &b->cub, &b->small, &b->trunc, &b->sides, &b->order, &b->flood})
        d->release();
    if (b->evInit)
        for (auto &e : b->ev)
            cudaEventDestroy(e);
    if (b->orderDone)
        cudaEventDestroy(b->orderDone);
    if (b->retriDone)
        cudaEventDestroy(b->retriDone);
    if (b->side) {
        cudaStreamDestroy(b->side);
        cudaEventDestroy(b->sideDone);
    }
    staged_wait(b);
    staged_release(b);
    if (b->stage) {
        cudaStreamDestroy(b->stage);
        cudaEventDestroy(b->stageEv);
    }
    pinned_mail_release(b->mail);
    delete b;
}

} // extern "C"

// ---------------------------------------------------------------------------------------------------
// batched booleans
// ---------------------------------------------------------------------------------------------------
struct sb_batch {
    std::vector<std::vector<double>> xyz;   // per pair: result vertices (empty unless kept and combined)
    std::vector<std::vector<uint32_t>> tris; // per pair: the triangles of the pair's operation
};

namespace {

// reuses a mesh handle for new inputs: the buffer grows when needed, everything derived is invalidated
sb_status mesh_reset(sb_mesh *m, const double *xyz, size_t nv, const uint32_t *tris, size_t nt, cudaStream_t s)
{
    if (nv > 0x7FFFFFFFu || nt > 0x2AAAAAAAu) {
        set_last_error("mesh too large");
        return SB_ERR_INVALID;
    }
    SB_CUDA_CHECK(m->buf.ensure(mesh_bytes((int)nv, (int)nt)));
    m->d = MeshDev{};
    m->d.nv = (int)nv;
    m->d.nt = (int)nt;
    Carve c;
    const size_t o_v = c.take<double>(nv * 3), o_t = c.take<uint32_t>(nt * 3);
    m->d.v = reinterpret_cast<double *>(m->buf.as<char>() + o_v);
    m->d.t = reinterpret_cast<uint32_t *>(m->buf.as<char>() + o_t);
    m->prepared = false;
    m->adjValid = false;
    m->rankPending = false;
    if (nv)
        SB_CUDA_CHECK(cudaMemcpyAsync(m->d.v, xyz, sizeof(double) * 3 * nv, cudaMemcpyHostToDevice, s));
    if (nt)
        SB_CUDA_CHECK(cudaMemcpyAsync(m->d.t, tris, sizeof(uint32_t) * 3 * nt, cudaMemcpyHostToDevice, s));
    return mesh_validate(m, s);
}

} // namespace

extern "C" {

constexpr int kMaxWorkers = 64;
constexpr size_t kTuneChunk = 64; // pairs per calibration run of the worker-count autotuner

sb_status sb_batch_combine(size_t n, const double *xyz_a, const uint64_t *v_off_a, const uint32_t *tris_a,
                           const uint64_t *t_off_a, const double *xyz_b, const uint64_t *v_off_b,
                           const uint32_t *tris_b, const uint64_t *t_off_b, const int32_t *ops,
                           const sb_options *opts, int32_t workers, int32_t *statuses, sb_batch **out)
{
    if (out)
        *out = nullptr;
    if (!statuses || (n && (!xyz_a || !v_off_a || !tris_a || !t_off_a || !xyz_b || !v_off_b || !tris_b || !t_off_b ||
                            !ops)))
        return SB_ERR_INVALID;
    return guarded([&]() -> sb_status {
        sb_options base;
        sb_default_options(&base);
        if (opts)
            base = *opts;
        std::unique_ptr<sb_batch> keep(out ? new sb_batch : nullptr);
        if (keep) {
            keep->xyz.resize(n);
            keep->tris.resize(n);
        }
        // pairs [next, end) go to the workers of the current run
        std::atomic<size_t> next{0};
        size_t end = n;
        std::vector<sb_status> setup(kMaxWorkers, SB_OK);
        // the largest pair's inputs, for the workers' pinned staging buffers
        size_t inMax = 0;
        for (size_t i = 0; i < n; ++i)
            inMax = std::max(inMax, 24 * (size_t)(v_off_a[i + 1] - v_off_a[i] + v_off_b[i + 1] - v_off_b[i]) +
                                        12 * (size_t)(t_off_a[i + 1] - t_off_a[i] + t_off_b[i + 1] - t_off_b[i]) + 64);
        // a worker's state lives across the runs of one call (the autotuner's calibration runs and the main
        // run): a non-blocking stream, a reusable pair of meshes and one boolean handle, a pinned staging
        // buffer for uploads and result reads (pageable copies go through the driver's staging path, which
        // serialises the workers' streams)
        struct Worker {
            cudaStream_t s = nullptr;
            sb_mesh *ma = nullptr, *mb = nullptr;
            sb_boolean *x = nullptr;
            char *stage = nullptr;
            size_t stageBytes = 0;
            bool ready = false;
        };
        std::vector<Worker> wk(kMaxWorkers);
        struct WorkersGone { // releases every worker's state however the call ends
            std::vector<Worker> &wk;
            ~WorkersGone()
            {
                for (Worker &k : wk) {
                    if (k.x)
                        sb_boolean_destroy(k.x);
                    sb_mesh_destroy(k.ma);
                    sb_mesh_destroy(k.mb);
                    if (k.s)
                        cudaStreamDestroy(k.s);
                    if (k.stage)
                        cudaFreeHost(k.stage);
                }
            }
        } gone{wk};
        auto pairs = [&](int w) {
            Worker &k = wk[w];
            auto stageFor = [&](size_t bytes) -> bool {
                if (bytes <= k.stageBytes)
                    return true;
                if (k.stage)
                    cudaFreeHost(k.stage);
                k.stage = nullptr;
                k.stageBytes = 0;
                const size_t want = bytes + bytes / 4;
                if (cudaMallocHost((void **)&k.stage, want) != cudaSuccess) {
                    k.stage = nullptr;
                    return false;
                }
                k.stageBytes = want;
                return true;
            };
            sb_status st = SB_OK;
            if (!k.ready) {
                if (cudaStreamCreateWithFlags(&k.s, cudaStreamNonBlocking) != cudaSuccess)
                    st = SB_ERR_CUDA;
                if (st == SB_OK)
                    st = mesh_alloc(0, 0, &k.ma);
                if (st == SB_OK)
                    st = mesh_alloc(0, 0, &k.mb);
                sb_options o = base;
                o.stream = k.s;
                o.stage_results = 0; // the batch copies the results it keeps itself
                if (st == SB_OK)
                    st = sb_boolean_create(k.ma, k.mb, &o, &k.x);
                if (st == SB_OK && !stageFor(inMax))
                    st = SB_ERR_CUDA;
                k.ready = st == SB_OK;
            }
            setup[w] = st;
            cudaStream_t s = k.s;
            for (size_t i = next++; st == SB_OK && i < end; i = next++) {
                const int op = ops[i];
                sb_status r = (op < SB_UNION || op > SB_INTERSECT) ? SB_ERR_INVALID : SB_OK;
                const size_t nva = v_off_a[i + 1] - v_off_a[i], nta = t_off_a[i + 1] - t_off_a[i];
                const size_t nvb = v_off_b[i + 1] - v_off_b[i], ntb = t_off_b[i + 1] - t_off_b[i];
                // staged inputs: A's vertices, B's vertices, A's triangles, B's triangles
                double *sva = reinterpret_cast<double *>(k.stage), *svb = sva + 3 * nva;
                uint32_t *sta = reinterpret_cast<uint32_t *>(svb + 3 * nvb), *stb = sta + 3 * nta;
                std::memcpy(sva, xyz_a + 3 * v_off_a[i], 24 * nva);
                std::memcpy(svb, xyz_b + 3 * v_off_b[i], 24 * nvb);
                std::memcpy(sta, tris_a + 3 * t_off_a[i], 12 * nta);
                std::memcpy(stb, tris_b + 3 * t_off_b[i], 12 * ntb);
                if (r == SB_OK)
                    r = mesh_reset(k.ma, sva, nva, sta, nta, s);
                if (r == SB_OK)
                    r = mesh_reset(k.mb, svb, nvb, stb, ntb, s);
                if (r == SB_OK)
                    r = sb_combine(k.x, nullptr);
                statuses[i] = r;
                if (keep && r == SB_OK) {
                    const size_t nv = k.x->nNewV, nt = k.x->nFetch[op];
                    sb_status q = stageFor(24 * nv + 12 * nt + 64) ? SB_OK : SB_ERR_CUDA;
                    double *rv = reinterpret_cast<double *>(k.stage);
                    uint32_t *rt = reinterpret_cast<uint32_t *>(rv + 3 * nv);
                    if (q == SB_OK && nv &&
                        cudaMemcpyAsync(rv, k.x->d_newV, 24 * nv, cudaMemcpyDeviceToHost, s) != cudaSuccess)
                        q = SB_ERR_CUDA;
                    if (q == SB_OK && nt &&
                        cudaMemcpyAsync(rt, k.x->d_fetch[op], 12 * nt, cudaMemcpyDeviceToHost, s) != cudaSuccess)
                        q = SB_ERR_CUDA;
                    if (q == SB_OK && cudaStreamSynchronize(s) != cudaSuccess)
                        q = SB_ERR_CUDA;
                    if (q == SB_OK) {
                        keep->xyz[i].assign(rv, rv + 3 * nv);
                        keep->tris[i].assign(rt, rt + 3 * nt);
                    }
                    if (q != SB_OK)
                        statuses[i] = q;
                }
            }
        };
        auto work = [&](int w) {
            try {
                pairs(w);
            } catch (...) {
                setup[w] = SB_ERR_INVALID;
            }
        };
        // one run: W workers over pairs [begin, stop)
        auto run = [&](size_t begin, size_t stop, int W) -> sb_status {
            next = begin;
            end = stop;
            std::vector<std::thread> pool;
            for (int w = 1; w < W; ++w)
                pool.emplace_back(work, w);
            work(0);
            for (auto &t : pool)
                t.join();
            for (int w = 0; w < W; ++w)
                if (setup[w] != SB_OK)
                    return setup[w];
            return SB_OK;
        };
        size_t done = 0;
        int W = workers > 0 ? std::min(workers, kMaxWorkers) : 8;
        if (workers <= 0 && n >= 8 * kTuneChunk) {
            // autotune: successive chunks of pairs (kept as results) on each candidate worker count, timed on
            // the host; the rest runs with the fastest
            double best = 0.0;
            for (int cand : {4, 8, 16}) {
                const auto t0 = std::chrono::steady_clock::now();
                const sb_status r = run(done, done + kTuneChunk, cand);
                const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
                if (r != SB_OK)
                    return r;
                done += kTuneChunk;
                if (best == 0.0 || dt < best) {
                    best = dt;
                    W = cand;
                }
            }
        }
        W = (int)std::max<int64_t>(1, std::min<int64_t>(W, (int64_t)(n - done)));
        if (done < n) {
            const sb_status r = run(done, n, W);
            if (r != SB_OK)
                return r;
        }
        if (out)
            *out = keep.release();
        return SB_OK;
    });
}

sb_status sb_batch_result_size(const sb_batch *b, size_t i, size_t *n_vertices, size_t *n_triangles)
{
    if (!b || i >= b->xyz.size() || !n_vertices || !n_triangles)
        return SB_ERR_INVALID;
    *n_vertices = b->xyz[i].size() / 3;
    *n_triangles = b->tris[i].size() / 3;
    return SB_OK;
}

sb_status sb_batch_result(const sb_batch *b, size_t i, double *xyz, uint32_t *tris)
{
    if (!b || i >= b->xyz.size() || (!xyz && !b->xyz[i].empty()) || (!tris && !b->tris[i].empty()))
        return SB_ERR_INVALID;
    std::copy(b->xyz[i].begin(), b->xyz[i].end(), xyz);
    std::copy(b->tris[i].begin(), b->tris[i].end(), tris);
    return SB_OK;
}

void sb_batch_destroy(sb_batch *b) { delete b; }

// page-locked host blocks, cached by size (a block serves requests down to half its size)
namespace {
struct HostCache {
    std::mutex mu;
    std::multimap<size_t, void *> free;
    std::unordered_map<void *, size_t> live;
    size_t cached = 0;
};
HostCache g_host;
constexpr size_t kHostCacheBytes = 2ull << 30;
} // namespace

sb_status sb_host_alloc(size_t bytes, void **ptr)
{
    if (!ptr)
        return SB_ERR_INVALID;
    *ptr = nullptr;
    const size_t want = std::max<size_t>(((bytes + 65535) >> 16) << 16, 65536);
    {
        std::lock_guard<std::mutex> lk(g_host.mu);
        auto it = g_host.free.lower_bound(want);
        if (it != g_host.free.end() && it->first <= 2 * want) {
            *ptr = it->second;
            g_host.live[it->second] = it->first;
            g_host.cached -= it->first;
            g_host.free.erase(it);
            return SB_OK;
        }
    }
    void *p = nullptr;
    const cudaError_t e = cudaMallocHost(&p, want);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaMallocHost(result buffer)", __FILE__, __LINE__);
    std::lock_guard<std::mutex> lk(g_host.mu);
    g_host.live[p] = want;
    *ptr = p;
    return SB_OK;
}

void sb_host_free(void *ptr)
{
    if (!ptr)
        return;
    std::lock_guard<std::mutex> lk(g_host.mu);
    auto it = g_host.live.find(ptr);
    if (it == g_host.live.end())
        return;
    const size_t sz = it->second;
    g_host.live.erase(it);
    if (g_host.cached + sz <= kHostCacheBytes) {
        g_host.free.insert({sz, ptr});
        g_host.cached += sz;
    } else {
        cudaFreeHost(ptr);
    }
}

sb_status sb_adjoint(sb_boolean *b, const double *d_grad_result, double *d_grad_first, double *d_grad_second,
                     void *stream)
{
    sb_status r = check_fetchable(b);
    if (r != SB_OK)
        return r;
    if (b->status != SB_OK || !d_grad_result || !d_grad_first || !d_grad_second)
        return SB_ERR_INVALID;
    return guarded([&]() -> sb_status {
        const MeshDev &A = b->first->d, &B = b->second->d;
        if (b->nNewV > 0) {
            const int bs = 256;
            SB_COUNT(k_adjoint)<<<(unsigned)((b->nNewV + bs - 1) / bs), bs, 0, (cudaStream_t)stream>>>(
                b->nNewV, A.nv, B.nv, d_grad_result, b->d_newSrc, b->d_pairAB, b->d_pairPerm, A, B, d_grad_first,
                d_grad_second);
        }
        SB_CUDA_CHECK(cudaGetLastError());
        return SB_OK;
    });
}

} // extern "C"
