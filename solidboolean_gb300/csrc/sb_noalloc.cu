// Allocation-free re-triangulation of cut faces.
//
// Some callers cannot allocate device memory: code inside a framework that owns every device allocation
// through its own memory pool (a cudaMalloc behind its back breaks its accounting and can fail once the
// pool has taken the free memory), and real-time loops where a cudaMalloc or cudaFree could stall or
// synchronise the device. For them sb_retriangulate_faces_noalloc runs the same per-face kernel as
// sb_combine (k_faces, sb_faces.cu) with its per-face workspace taken from one file-scope static device
// array of fixed size instead of from a cudaMalloc'd buffer. The caller passes every input and output.
//
// Rules of use:
//   * the workspace is kNoAllocScratchBytes (64 MiB) per device; every GPU that loads the library holds it
//     until the process exits;
//   * size checks: a request whose fixed layout (per-face tables, per-segment keys) does not fit returns
//     SB_ERR_CAPACITY before any launch; the per-face workspace total is only known after a sizing pass
//     that runs on the GPU and writes into the shared array, so a request that fails that second check
//     returns SB_ERR_CAPACITY after the sizing pass, without running the re-triangulation;
//   * the call reads that total back and waits for its stream (cudaStreamSynchronize) before it launches
//     the re-triangulation;
//   * the first call on a device, with that device current, looks up the array's device address
//     (cudaGetSymbolAddress) and caches it per device: make that first call before any stream capture.
//     cudaDeviceReset, or anything else that destroys the primary context, invalidates the cached
//     address: do not call this entry point again in a process after that;
//   * all calls share the array and it keeps the previous call's contents (the parts that must start at
//     zero are cleared by each call): calls that can overlap on the GPU (different streams, or threads)
//     race and must be serialised by the caller;
//   * no cudaMalloc, cudaFree or allocating library routine is called (the prefix sum uses CUB with its
//     temporary storage carved from the same array).
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

#include <cub/cub.cuh>

#include "sb_common.cuh"
#include "sb_faces.cuh"
#include "sb_internal.h"

namespace sbg {

constexpr size_t kNoAllocScratchBytes = 64ull << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static std::mutex g_noalloc_mutex;
static void *g_noalloc_ptr[256];

// device address of the static array for the current device (set up once per device)
static sb_status noalloc_base(void **out)
{
    int dev = 0;
    SB_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256)
        return SB_ERR_INVALID;
    std::lock_guard<std::mutex> lk(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        SB_CUDA_CHECK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return SB_OK;
}

__global__ void k_na_setup(int nFaces, int nSeg, const int *__restrict__ segBegin, int triCap, int *faceSide,
                           int *faceTri, int *pairIdx, uint32_t *cornerTris, int *ptOff, int *triOff, int *edgeOff,
                           unsigned long long *scratchBytes, int *invalid)
{
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f < nSeg)
        pairIdx[f] = f;
    if (f > nFaces)
        return;
    if (f == nFaces) {
        ptOff[f] = 2 * nSeg;
        triOff[f] = nFaces * triCap;
        edgeOff[f] = 2 * nSeg;
        scratchBytes[f] = 0;
        if (segBegin[nFaces] != nSeg || segBegin[0] != 0)
            atomicOr(invalid, 1);
        return;
    }
    int b = segBegin[f], e = segBegin[f + 1];
    if (e < b || b < 0 || e > nSeg)
        atomicOr(invalid, 1);
    faceSide[f] = 0;
    faceTri[f] = f;
    cornerTris[3 * f] = 3u * f;
    cornerTris[3 * f + 1] = 3u * f + 1u;
    cornerTris[3 * f + 2] = 3u * f + 2u;
    ptOff[f] = 2 * b;
    triOff[f] = f * triCap;
    edgeOff[f] = 2 * b;
}

} // namespace sbg

using namespace sbg;

extern "C" sb_status sb_retriangulate_faces_noalloc(const double *d_corners, const int *d_seg_begin,
                                                    const double *d_segments, int n_faces, int n_segments,
                                                    int64_t weld_factor, int *d_tris, int tri_cap,
                                                    int *d_tri_count, double *d_points, int *d_point_count,
                                                    int *d_status, void *stream)
{
    if (n_faces < 0 || n_segments < 0 || tri_cap <= 0 || weld_factor <= 0)
        return SB_ERR_INVALID;
    if (n_faces == 0)
        return SB_OK;
    if (!d_corners || !d_seg_begin || !d_tris || !d_tri_count || !d_points || !d_point_count || !d_status ||
        (n_segments > 0 && !d_segments))
        return SB_ERR_INVALID;
    if ((long long)n_faces * tri_cap > 0x7FFFFFFFll || 2ll * n_segments > 0x7FFFFFFFll) {
        set_last_error("no-alloc retriangulation: sizes exceed 32-bit offsets");
        return SB_ERR_CAPACITY;
    }
    cudaStream_t s = (cudaStream_t)stream;
    void *basev = nullptr;
    sb_status r = noalloc_base(&basev);
    if (r != SB_OK)
        return r;
    char *base = (char *)basev;

    // fixed part of the layout inside the static array
    size_t scanBytes = 0;
    SB_CUDA_CHECK(cub::DeviceScan::ExclusiveSum(nullptr, scanBytes, (unsigned long long *)nullptr,
                                                (unsigned long long *)nullptr, n_faces + 1, s));
    Carve c;
    size_t o_hdr = c.take<int>(64);
    size_t o_scan = c.take<char>(scanBytes);
    size_t o_sb = c.take<unsigned long long>(n_faces + 1), o_so = c.take<unsigned long long>(n_faces + 1);
    size_t o_side = c.take<int>(n_faces + 1), o_tri = c.take<int>(n_faces + 1);
    size_t o_pidx = c.take<int>(n_segments + 1), o_ct = c.take<uint32_t>(3 * (size_t)n_faces);
    size_t o_po = c.take<int>(n_faces + 1), o_to = c.take<int>(n_faces + 1), o_eo = c.take<int>(n_faces + 1);
    size_t o_keys = c.take<Key>(2 * (size_t)n_segments + 1), o_edges = c.take<int>(4 * (size_t)n_segments + 2);
    size_t o_ne = c.take<int>(n_faces + 1);
    size_t o_c1 = c.take<int>(n_faces + 1), o_c2 = c.take<int>(n_faces + 1), o_c3 = c.take<int>(n_faces + 1);
    const size_t fixedBytes = c.off;
    if (fixedBytes > kNoAllocScratchBytes) {
        set_last_error("no-alloc retriangulation: " + std::to_string(n_faces) + " faces / " +
                       std::to_string(n_segments) + " segments exceed the 64 MiB workspace");
        return SB_ERR_CAPACITY;
    }
    int *hdr = (int *)(base + o_hdr);
    unsigned long long *scratchBytes = (unsigned long long *)(base + o_sb);
    unsigned long long *scratchOff = (unsigned long long *)(base + o_so);
    int *faceSide = (int *)(base + o_side), *faceTri = (int *)(base + o_tri), *pairIdx = (int *)(base + o_pidx);
    uint32_t *cornerTris = (uint32_t *)(base + o_ct);
    int *ptOff = (int *)(base + o_po), *triOff = (int *)(base + o_to), *edgeOff = (int *)(base + o_eo);
    // the header (validation flag) must start at zero; everything else is written before it is read
    SB_CUDA_CHECK(cudaMemsetAsync(hdr, 0, 64 * sizeof(int), s));
    int threads = std::max(n_faces + 1, n_segments);
    SB_COUNT(k_na_setup)<<<(threads + 255) / 256, 256, 0, s>>>(n_faces, n_segments, d_seg_begin, tri_cap, faceSide,
                                                                faceTri, pairIdx, cornerTris, ptOff, triOff, edgeOff,
                                                                scratchBytes, hdr);
    // the per-face workspace bounds, computed by the same routine sb_combine uses
    launch_face_sizes(n_faces, d_seg_begin, scratchBytes, (int *)(base + o_c1), (int *)(base + o_c2),
                      (int *)(base + o_c3), s);
    SB_CUDA_CHECK(cub::DeviceScan::ExclusiveSum(base + o_scan, scanBytes, scratchBytes, scratchOff, n_faces + 1, s));
    unsigned long long total = 0;
    int invalid = 0;
    SB_CUDA_CHECK(cudaMemcpyAsync(&total, scratchOff + n_faces, sizeof total, cudaMemcpyDeviceToHost, s));
    SB_CUDA_CHECK(cudaMemcpyAsync(&invalid, hdr, sizeof invalid, cudaMemcpyDeviceToHost, s));
    SB_CUDA_CHECK(cudaStreamSynchronize(s));
    if (invalid) {
        set_last_error("no-alloc retriangulation: seg_begin is not a CSR offset array of n_segments");
        return SB_ERR_INVALID;
    }
    const size_t workOff = (fixedBytes + 255) & ~size_t(255);
    if (workOff + total > kNoAllocScratchBytes) {
        set_last_error("no-alloc retriangulation: the faces need " + std::to_string(workOff + total) +
                       " bytes of workspace, more than the 64 MiB static array");
        return SB_ERR_CAPACITY;
    }
    FaceArgs fa;
    std::memset(&fa, 0, sizeof fa);
    fa.scratchCap = ~0ull; // the workspace total was checked against the static array above
    fa.A.v = const_cast<double *>(d_corners);
    fa.A.nv = 3 * n_faces;
    fa.A.t = cornerTris;
    fa.A.nt = n_faces;
    fa.B = fa.A;
    fa.nFaces = n_faces;
    fa.faceSide = faceSide;
    fa.faceTri = faceTri;
    fa.faceBegin = d_seg_begin;
    fa.pairIdx = pairIdx;
    fa.segs = d_segments;
    fa.factor = (double)weld_factor;
    fa.scratch = base + workOff;
    fa.scratchOff = scratchOff;
    fa.ptOff = ptOff;
    fa.triOff = triOff;
    fa.edgeOff = edgeOff;
    fa.cutPts = reinterpret_cast<d3 *>(d_points);
    fa.cutKeys = (Key *)(base + o_keys);
    fa.faceTris = d_tris;
    fa.faceEdges = (int *)(base + o_edges);
    fa.faceStatus = d_status;
    fa.faceNpts = d_point_count;
    fa.faceNtris = d_tri_count;
    fa.faceNedges = (int *)(base + o_ne);
    launch_faces(fa, s);
    SB_CUDA_CHECK(cudaGetLastError());
    return SB_OK;
}
