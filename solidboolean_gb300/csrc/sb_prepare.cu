// Mesh preparation on the GPU (the counterpart of SolidMesh::prepare, src/solidmesh.cpp:42-76).
//
// The reference builds unit normals, per-triangle AABBs and a top-down AABB tree. Here:
//   * per-triangle AABBs (exact FP64 min/max, plus a round-to-nearest FP32 copy for the filtered tests);
//   * an LBVH: 24-bit Morton codes of the FP32 box centres, a radix sort, Karras' hierarchy construction
//     (one thread per internal node) and a bottom-up refit in which the second child to arrive at a node
//     (atomic counter) writes the union box;
//   * unit normals are not stored: the kernels that need one recompute it with the reference's formula.
// The reference tree's leaf order, needed only to reproduce its per-face pair order, is built by
// sb_refrank.cu.
#include <cub/cub.cuh>

#include "sb_common.cuh"
#include "sb_hash.cuh"
#include "sb_internal.h"

namespace sbg {

// FP32 vertex copies; threads 0-11 also reset the 12 words that k_tri_boxes accumulates: the centre bounds
// (min keys at all ones, max keys at zero), two unused words, and the per-axis largest |coordinate| (zero)
constexpr int kBoundWords = 12;
__global__ void k_vertices_f32(int nv, const double *__restrict__ v, float4 *__restrict__ vf, unsigned int *bounds)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kBoundWords)
        bounds[i] = i < 3 ? 0xFFFFFFFFu : 0u;
    if (i >= nv)
        return;
    vf[i] = make_float4(__double2float_rn(v[3 * i]), __double2float_rn(v[3 * i + 1]),
                        __double2float_rn(v[3 * i + 2]), 0.0f);
}

// Per-triangle box, updated vertex by vertex like AxisAlignedBoudingBox::update
// (src/axisalignedboundingbox.h:31-41), and the FP32 box centre used for the Morton code.
__global__ void k_tri_boxes(int nt, const double *__restrict__ v, const uint32_t *__restrict__ t,
                            double *__restrict__ box64, float *__restrict__ box32, float *__restrict__ cen,
                            unsigned int *__restrict__ bounds)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    float c[3] = {0.f, 0.f, 0.f};
    unsigned int amax[3] = {0u, 0u, 0u}; // FP32 bits of the largest |coordinate|, rounded up
    bool valid = i < nt;
    if (valid) {
        double lo[3] = {kDblMax, kDblMax, kDblMax};
        double hi[3] = {-kDblMax, -kDblMax, -kDblMax};
        for (int k = 0; k < 3; ++k) {
            const double *p = v + 3 * (size_t)t[3 * i + k];
            for (int a = 0; a < 3; ++a) {
                double x = p[a];
                if (x > hi[a])
                    hi[a] = x;
                if (x < lo[a])
                    lo[a] = x;
            }
        }
        for (int a = 0; a < 3; ++a) {
            box64[6 * (size_t)i + a] = lo[a];
            box64[6 * (size_t)i + 3 + a] = hi[a];
            float l = __double2float_rn(lo[a]), h = __double2float_rn(hi[a]);
            box32[6 * (size_t)i + a] = l;
            box32[6 * (size_t)i + 3 + a] = h;
            c[a] = 0.5f * l + 0.5f * h;
            cen[3 * (size_t)i + a] = c[a];
            amax[a] = __float_as_uint(__double2float_ru(fmax(fabs(lo[a]), fabs(hi[a]))));
        }
    }
    // block-wide min/max of the centres, then one atomic per block and axis (ordered-int encoding)
    __shared__ unsigned int smin[3][32], smax[3][32], sabs[3][32];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int a = 0; a < 3; ++a) {
        unsigned int u = __float_as_uint(c[a]);
        unsigned int o = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
        unsigned int mn = valid ? o : 0xFFFFFFFFu, mx = valid ? o : 0u;
        unsigned int am = amax[a]; // non-negative floats order as their bits
        for (int s = 16; s > 0; s >>= 1) {
            mn = min(mn, __shfl_xor_sync(0xFFFFFFFFu, mn, s));
            mx = max(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, s));
            am = max(am, __shfl_xor_sync(0xFFFFFFFFu, am, s));
        }
        if (lane == 0) {
            smin[a][warp] = mn;
            smax[a][warp] = mx;
            sabs[a][warp] = am;
        }
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        int a = threadIdx.x;
        unsigned int mn = 0xFFFFFFFFu, mx = 0u, am = 0u;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            mn = min(mn, smin[a][w]);
            mx = max(mx, smax[a][w]);
            am = max(am, sabs[a][w]);
        }
        atomicMin(bounds + a, mn);
        atomicMax(bounds + 3 + a, mx);
        atomicMax(bounds + 8 + a, am);
    }
}

__device__ __forceinline__ float ord_to_float(unsigned int o)
{
    unsigned int u = (o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o;
    return __uint_as_float(u);
}

__device__ __forceinline__ uint32_t expand10(uint32_t x)
{
    x &= 0x3FFu;
    x = (x | (x << 16)) & 0x030000FFu;
    x = (x | (x << 8)) & 0x0300F00Fu;
    x = (x | (x << 4)) & 0x030C30C3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

// Morton code bits per axis. Eight (a 24-bit code, three radix passes instead of four for ten bits): the
// results do not depend on the LBVH's leaf order, only the candidate search's speed does, and at 2^8 cells per
// axis a surface mesh of a few hundred thousand triangles still holds about one or two triangles per cell
// (equal codes are split by triangle index).
constexpr int kMortonAxisBits = 8;
constexpr int kMortonBits = 3 * kMortonAxisBits;

__global__ void k_morton(int nt, const float *__restrict__ cen, const unsigned int *__restrict__ bounds,
                         uint32_t *__restrict__ code, int *__restrict__ idx)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt)
        return;
    uint32_t q[3];
    for (int a = 0; a < 3; ++a) {
        float lo = ord_to_float(bounds[a]), hi = ord_to_float(bounds[3 + a]);
        float ext = hi - lo;
        float u = ext > 0.f ? (cen[3 * (size_t)i + a] - lo) / ext : 0.f;
        int k = (int)(u * (float)(1 << kMortonAxisBits));
        q[a] = (uint32_t)min(max(k, 0), (1 << kMortonAxisBits) - 1);
    }
    code[i] = (expand10(q[0]) << 2) | (expand10(q[1]) << 1) | expand10(q[2]);
    idx[i] = i;
}

// common-prefix length of the (code, index) keys of leaves i and j; -1 outside [0, n)
__device__ __forceinline__ int lbvh_delta(const uint32_t *code, int n, int i, int j)
{
    if (j < 0 || j >= n)
        return -1;
    uint32_t a = code[i], b = code[j];
    if (a == b)
        return 32 + __clz((unsigned)(i ^ j));
    return __clz(a ^ b);
}

// Karras 2012, "Maximizing parallelism in the construction of BVHs, octrees and k-d trees".
__global__ void k_karras(int n, const uint32_t *__restrict__ code, int2 *__restrict__ child, int *__restrict__ parent)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1)
        return;
    int d = (lbvh_delta(code, n, i, i + 1) - lbvh_delta(code, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = lbvh_delta(code, n, i, i - d);
    int lmax = 2;
    while (lbvh_delta(code, n, i, i + lmax * d) > dmin)
        lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (lbvh_delta(code, n, i, i + (l + t) * d) > dmin)
            l += t;
    int j = i + l * d;
    int dnode = lbvh_delta(code, n, i, j);
    int s = 0;
    int div = 2;
    int t = (l + div - 1) / div;
    while (true) {
        if (lbvh_delta(code, n, i, i + (s + t) * d) > dnode)
            s += t;
        if (t == 1)
            break;
        div <<= 1;
        t = (l + div - 1) / div;
    }
    int gamma = i + s * d + min(d, 0);
    int lo = min(i, j), hi = max(i, j);
    int left = (lo == gamma) ? ~gamma : gamma;
    int right = (hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
    child[i] = make_int2(left, right);
    parent[left >= 0 ? left : (n - 1) + ~left] = i;
    parent[right >= 0 ? right : (n - 1) + ~right] = i;
}

// Arrival at a node of the climb: an atomic add with acquire-release semantics at device scope. The release
// publishes the box this thread wrote for the child it climbed from; the acquire makes the sibling's box,
// written by the thread that arrived first, visible to the loads that follow.
__device__ __forceinline__ int arrive_acq_rel(int *flag)
{
    int old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], 1;" : "=r"(old) : "l"(flag) : "memory");
    return old;
}

// Bottom-up refit: one thread per leaf climbs while it is the second to reach a node, and writes the node's
// box as the union of the box it carries (its own subtree's, in registers) and the sibling's (one load of six
// doubles). The FP32 copy rounds the FP64 union outward (down for the low corner, up for the high corner);
// directed rounding is monotone, so this equals the union of the children's outward-rounded boxes.
__global__ void k_refit(int n, const int *__restrict__ leafTri, const double *__restrict__ box64,
                        const int2 *__restrict__ child, const int *__restrict__ parent, int *flags, double *nbox64,
                        float *nbox32)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double m[6];
    {
        const int tri = leafTri[i];
        for (int k = 0; k < 6; ++k)
            m[k] = box64[6 * (size_t)tri + k];
    }
    int cur = ~i; // child id of leaf i
    int node = parent[(n - 1) + i];
    while (node >= 0) {
        // the hierarchy does not change during the refit: the node's children and parent are loaded before
        // the arrival, so that their latency overlaps the atomic's (two dependent round trips per level, the
        // arrival and the sibling's box, instead of four)
        const int2 ch = child[node];
        const int up = parent[node];
        if (arrive_acq_rel(flags + node) == 0)
            return;
        const int sib = ch.x == cur ? ch.y : ch.x;
        const double *sb = sib < 0 ? box64 + 6 * (size_t)__ldcg(leafTri + ~sib) : nbox64 + 6 * (size_t)sib;
        for (int k = 0; k < 3; ++k) {
            m[k] = fmin(m[k], __ldcg(sb + k));
            m[3 + k] = fmax(m[3 + k], __ldcg(sb + 3 + k));
        }
        for (int k = 0; k < 3; ++k) {
            nbox64[6 * (size_t)node + k] = m[k];
            nbox64[6 * (size_t)node + 3 + k] = m[3 + k];
        }
        reinterpret_cast<float4 *>(nbox32)[2 * (size_t)node] =
            make_float4(__double2float_rd(m[0]), __double2float_rd(m[1]), __double2float_rd(m[2]), 0.f);
        reinterpret_cast<float4 *>(nbox32)[2 * (size_t)node + 1] =
            make_float4(__double2float_ru(m[3]), __double2float_ru(m[4]), __double2float_ru(m[5]), 0.f);
        cur = node;
        node = up;
    }
}

static inline int blocks_for(size_t n, int bs) { return (int)((n + bs - 1) / bs); }

// Edge adjacency of the input triangles: every directed edge (a -> b) into a table that keeps its first
// triangle in index order; then each edge's reverse (b -> a) looked up. This is the half-edge map the
// reference builds over the arrangement (src/solidboolean.cpp:167-239) restricted to one input mesh, so the
// grouping can read the twins of uncut triangles directly instead of hashing all of their half-edges.
static uint32_t adj_capacity(int nt)
{
    uint32_t p = 1024;
    while (p < 2ull * 3ull * (uint64_t)nt)
        p <<= 1;
    return p;
}

__global__ void k_adj_insert(int nt, const uint32_t *__restrict__ t, uint64_t *keys, int *vals, uint32_t mask)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt)
        return;
    const uint32_t v[3] = {t[3 * (size_t)i], t[3 * (size_t)i + 1], t[3 * (size_t)i + 2]};
    for (int k = 0; k < 3; ++k)
        u64map_insert_min(keys, vals, mask, he_key(v[k], v[(k + 1) % 3]), i);
}

__global__ void k_adj_find(int nt, const uint32_t *__restrict__ t, const uint64_t *__restrict__ keys,
                           const int *__restrict__ vals, uint32_t mask, int *adj, int *adjDup)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt)
        return;
    const uint32_t v[3] = {t[3 * (size_t)i], t[3 * (size_t)i + 1], t[3 * (size_t)i + 2]};
    if (v[0] == v[1] && v[1] == v[2])
        atomicAdd(adjDup, 1); // (a, a, a) holds the edge (a, a) three times
    for (int k = 0; k < 3; ++k) {
        const uint32_t a = v[k], b = v[(k + 1) % 3];
        if (u64map_find(keys, vals, mask, he_key(a, b)) != i)
            atomicAdd(adjDup, 1);
        adj[3 * (size_t)i + k] = u64map_find(keys, vals, mask, he_key(b, a));
    }
}

// What the phases of one mesh's preparation pass on to each other.
struct PrepState {
    bool active = false; // the mesh has triangles and was not prepared
    bool fork = false;   // the reference leaf order is built (on the mesh's second stream)
    char *tb = nullptr;  // temporaries
    size_t t_ak = 0, t_av = 0;
    uint32_t adjCap = 0;
    cudaStream_t s = nullptr;
};

sb_status mesh_order_after(sb_mesh *m, cudaStream_t s)
{
    if (m->rankPending && m->aux)
        SB_CUDA_CHECK(cudaStreamWaitEvent(s, m->auxJoin, 0));
    if (m->readyEv)
        SB_CUDA_CHECK(cudaStreamWaitEvent(s, m->readyEv, 0));
    return SB_OK;
}

// Phase 1: layout, FP32 vertices, triangle boxes, Morton codes and order; the second stream forks here.
static sb_status prepare_begin(sb_mesh *m, int order_mode, cudaStream_t s, PrepState &ps)
{
    MeshDev &d = m->d;
    const int nt = d.nt;
    ps = PrepState{};
    ps.s = s;
    {
        // the buffers below may still be read by a previous preparation's work
        const sb_status r = mesh_order_after(m, s);
        if (r != SB_OK)
            return r;
    }
    if (nt <= 0) {
        m->prepared = true;
        return SB_OK;
    }
    ps.active = true;
    // layout of the prepared arrays after the input arrays (v, t) already in m->buf
    Carve c;
    size_t o_v = c.take<double>((size_t)d.nv * 3);
    size_t o_t = c.take<uint32_t>((size_t)nt * 3);
    size_t o_vf = c.take<float4>((size_t)d.nv);
    size_t o_b64 = c.take<double>((size_t)nt * 6);
    size_t o_b32 = c.take<float>((size_t)nt * 6);
    size_t o_mc = c.take<uint32_t>((size_t)nt);
    size_t o_lt = c.take<int>((size_t)nt);
    size_t o_ch = c.take<int2>((size_t)(nt > 1 ? nt - 1 : 1));
    size_t o_pa = c.take<int>((size_t)(2 * nt));
    size_t o_n32 = c.take<float>((size_t)(nt > 1 ? nt - 1 : 1) * 8);
    size_t o_n64 = c.take<double>((size_t)(nt > 1 ? nt - 1 : 1) * 6);
    size_t o_fl = c.take<int>((size_t)(nt > 1 ? nt - 1 : 1));
    size_t o_rk = c.take<int>((size_t)nt);
    size_t o_adj = c.take<int>((size_t)nt * 3);
    size_t o_ad = c.take<int>(1);
    (void)o_v;
    (void)o_t;
    if (m->buf.bytes < c.off) {
        // inputs live at the front of buf; grow while keeping them
        DevBuf nb;
        SB_CUDA_CHECK(nb.ensure(c.off));
        SB_CUDA_CHECK(cudaMemcpyAsync(nb.ptr, m->buf.ptr, o_vf, cudaMemcpyDeviceToDevice, s));
        SB_CUDA_CHECK(cudaStreamSynchronize(s));
        m->buf.release();
        m->buf = nb;
        m->adjValid = false;
        d.v = m->buf.as<double>();
        d.t = reinterpret_cast<uint32_t *>(m->buf.as<char>() + o_t);
    }
    char *base = m->buf.as<char>();
    d.vf = reinterpret_cast<float4 *>(base + o_vf);
    d.box64 = reinterpret_cast<double *>(base + o_b64);
    d.box32 = reinterpret_cast<float *>(base + o_b32);
    d.morton = reinterpret_cast<uint32_t *>(base + o_mc);
    d.leafTri = reinterpret_cast<int *>(base + o_lt);
    d.child = reinterpret_cast<int2 *>(base + o_ch);
    d.parent = reinterpret_cast<int *>(base + o_pa);
    d.nbox32 = reinterpret_cast<float *>(base + o_n32);
    d.nbox64 = reinterpret_cast<double *>(base + o_n64);
    d.flags = reinterpret_cast<int *>(base + o_fl);
    d.rank = reinterpret_cast<int *>(base + o_rk);
    d.adj = reinterpret_cast<int *>(base + o_adj);
    d.adjDup = reinterpret_cast<int *>(base + o_ad);

    // temporaries: centres, bounds, unsorted keys/indices, CUB scratch
    size_t sortBytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, sortBytes, (uint32_t *)nullptr, (uint32_t *)nullptr, (int *)nullptr,
                                    (int *)nullptr, nt, 0, kMortonBits, s);
    Carve tc;
    size_t t_cen = tc.take<float>((size_t)nt * 3);
    size_t t_bnd = tc.take<unsigned int>(kBoundWords);
    size_t t_key = tc.take<uint32_t>((size_t)nt);
    size_t t_idx = tc.take<int>((size_t)nt);
    size_t t_cub = tc.take<char>(sortBytes);
    const uint32_t adjCap = adj_capacity(nt);
    size_t t_ak = m->adjValid ? 0 : tc.take<uint64_t>(adjCap);
    size_t t_av = m->adjValid ? 0 : tc.take<int>(adjCap);
    SB_CUDA_CHECK(m->tmp.ensure(tc.off));
    char *tb = m->tmp.as<char>();
    float *cen = reinterpret_cast<float *>(tb + t_cen);
    unsigned int *bounds = reinterpret_cast<unsigned int *>(tb + t_bnd);
    uint32_t *keyIn = reinterpret_cast<uint32_t *>(tb + t_key);
    d.absMax = bounds + 8; // the leaf order's fixed-point grids
    int *idxIn = reinterpret_cast<int *>(tb + t_idx);

    const int BS = 256;
    SB_COUNT(k_vertices_f32)<<<blocks_for(std::max(d.nv, 8), BS), BS, 0, s>>>(d.nv, d.v, d.vf, bounds);
    SB_COUNT(k_tri_boxes)<<<blocks_for(nt, BS), BS, 0, s>>>(nt, d.v, d.t, d.box64, d.box32, cen, bounds);
    SB_COUNT(k_morton)<<<blocks_for(nt, BS), BS, 0, s>>>(nt, cen, bounds, keyIn, idxIn);
    SB_CUDA_CHECK(cub::DeviceRadixSort::SortPairs(tb + t_cub, sortBytes, keyIn, d.morton, idxIn, d.leafTri, nt, 0,
                                                  kMortonBits, s));
    // The reference leaf order needs only the boxes and the Morton order: it runs on a second stream while
    // this one builds and refits the LBVH.
    const bool fork = order_mode == SB_ORDER_REFERENCE;
    ps.fork = fork;
    ps.tb = tb;
    ps.t_ak = t_ak;
    ps.t_av = t_av;
    ps.adjCap = adjCap;
    if (fork) {
        if (!m->aux) {
            SB_CUDA_CHECK(cudaStreamCreateWithFlags(&m->aux, cudaStreamNonBlocking));
            SB_CUDA_CHECK(cudaEventCreateWithFlags(&m->auxFork, cudaEventDisableTiming));
            SB_CUDA_CHECK(cudaEventCreateWithFlags(&m->auxJoin, cudaEventDisableTiming));
        }
        SB_CUDA_CHECK(cudaEventRecord(m->auxFork, s));
        SB_CUDA_CHECK(cudaStreamWaitEvent(m->aux, m->auxFork, 0));
    }
    return SB_OK;
}

// Phase 2: the reference leaf order, issued on the mesh's second stream (waits there for phase 1).
static sb_status prepare_rank(sb_mesh *m, bool waitRank, PrepState &ps)
{
    if (!ps.active || !ps.fork)
        return SB_OK;
    m->d.rankValid = false;
    const sb_status st = build_reference_rank(m, m->aux, waitRank);
    SB_CUDA_CHECK(cudaEventRecord(m->auxJoin, m->aux));
    return st;
}

// Phase 3: LBVH hierarchy and refit, input edge adjacency; with waitRank the main stream joins the leaf order.
static sb_status prepare_end(sb_mesh *m, bool waitRank, PrepState &ps)
{
    if (!ps.active)
        return SB_OK;
    MeshDev &d = m->d;
    const int nt = d.nt;
    cudaStream_t s = ps.s;
    char *tb = ps.tb;
    const uint32_t adjCap = ps.adjCap;
    const size_t t_ak = ps.t_ak, t_av = ps.t_av;
    const int BS = 256;
    if (nt > 1) {
        SB_CUDA_CHECK(cudaMemsetAsync(d.parent, 0xFF, sizeof(int) * 2 * (size_t)nt, s));
        SB_CUDA_CHECK(cudaMemsetAsync(d.flags, 0, sizeof(int) * (size_t)(nt - 1), s));
        SB_COUNT(k_karras)<<<blocks_for(nt - 1, BS), BS, 0, s>>>(nt, d.morton, d.child, d.parent);
        SB_COUNT(k_refit)<<<blocks_for(nt, BS), BS, 0, s>>>(nt, d.leafTri, d.box64, d.child, d.parent, d.flags, d.nbox64,
                                                  d.nbox32);
        d.root = 0;
    } else {
        d.root = ~0;
    }
    if (!m->adjValid) {
        uint64_t *ak = reinterpret_cast<uint64_t *>(tb + t_ak);
        int *av = reinterpret_cast<int *>(tb + t_av);
        SB_CUDA_CHECK(cudaMemsetAsync(ak, 0xFF, sizeof(uint64_t) * adjCap, s));
        SB_CUDA_CHECK(cudaMemsetAsync(av, 0x7F, sizeof(int) * adjCap, s)); // above any triangle index
        SB_CUDA_CHECK(cudaMemsetAsync(d.adjDup, 0, sizeof(int), s));
        SB_COUNT(k_adj_insert)<<<blocks_for(nt, BS), BS, 0, s>>>(nt, d.t, ak, av, adjCap - 1);
        SB_COUNT(k_adj_find)<<<blocks_for(nt, BS), BS, 0, s>>>(nt, d.t, ak, av, adjCap - 1, d.adj, d.adjDup);
        m->adjValid = true;
    }
    SB_CUDA_CHECK(cudaGetLastError());
    if (ps.fork && waitRank)
        SB_CUDA_CHECK(cudaStreamWaitEvent(s, m->auxJoin, 0));
    if (!ps.fork)
        d.rankValid = false;
    if (!m->readyEv)
        SB_CUDA_CHECK(cudaEventCreateWithFlags(&m->readyEv, cudaEventDisableTiming));
    SB_CUDA_CHECK(cudaEventRecord(m->readyEv, s));
    m->prepared = true;
    return SB_OK;
}

sb_status prepare_mesh(sb_mesh *m, int order_mode, cudaStream_t s, bool waitRank)
{
    PrepState ps;
    sb_status r = prepare_begin(m, order_mode, s, ps);
    if (r != SB_OK || !ps.active)
        return r;
    if (waitRank) {
        // the leaf-order build synchronises the host: issue the LBVH first
        r = prepare_end(m, false, ps);
        if (r == SB_OK)
            r = prepare_rank(m, true, ps);
        if (r == SB_OK && ps.fork)
            SB_CUDA_CHECK(cudaStreamWaitEvent(s, m->auxJoin, 0));
        return r;
    }
    r = prepare_rank(m, false, ps);
    if (r != SB_OK)
        return r;
    return prepare_end(m, false, ps);
}

sb_status prepare_meshes(sb_mesh *a, cudaStream_t sa, sb_mesh *b, cudaStream_t sb, int order_mode)
{
    // the leaf orders are the longer path: both are issued before either LBVH
    PrepState pa, pb;
    sb_status r = prepare_begin(a, order_mode, sa, pa);
    if (r == SB_OK)
        r = prepare_begin(b, order_mode, sb, pb);
    if (r == SB_OK)
        r = prepare_rank(a, false, pa);
    if (r == SB_OK)
        r = prepare_rank(b, false, pb);
    if (r == SB_OK)
        r = prepare_end(a, false, pa);
    if (r == SB_OK)
        r = prepare_end(b, false, pb);
    return r;
}

} // namespace sbg
