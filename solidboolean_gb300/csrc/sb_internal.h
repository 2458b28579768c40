// Internal host-side structures shared by the .cu translation units (not part of the C ABI).
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/solidboolean_gb300.h"

namespace sbg {

sb_status cuda_fail(cudaError_t e, const char *expr, const char *file, int line);
void set_last_error(const std::string &msg);

// Device memory block owned by a mesh or a boolean. Grows by reallocation only (never shrinks).
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t need);
    void release();
    template <class T> T *as() const { return reinterpret_cast<T *>(ptr); }
};

// Bump allocator over one DevBuf; offsets are 256-byte aligned.
struct Carve {
    size_t off = 0;
    template <class T> size_t take(size_t count)
    {
        size_t o = off;
        off += (count * sizeof(T) + 255) & ~size_t(255);
        return o;
    }
};

// LBVH over the triangles of one mesh. Internal nodes 0..n-2 (root 0); a child index c >= 0 is an internal
// node and c < 0 is the leaf ~c (position in Morton order). FP32 node boxes are rounded outward (they only
// prune); FP64 node boxes are exact unions (plain FP64 form).
struct MeshDev {
    int nv = 0, nt = 0;
    double *v = nullptr;      // [nv*3] FP64 xyz
    uint32_t *t = nullptr;    // [nt*3]
    float4 *vf = nullptr;     // [nv] FP32 copy (round to nearest) for the filtered predicates
    double *box64 = nullptr;  // [nt*6] lo xyz, hi xyz
    float *box32 = nullptr;   // [nt*6] round-to-nearest copy of box64
    uint32_t *morton = nullptr;
    int *leafTri = nullptr;   // [nt] triangle at each Morton-ordered leaf
    int2 *child = nullptr;    // [nt-1] (left, right)
    int *parent = nullptr;    // [2*nt-1]: internal nodes then leaves (offset nt-1)
    float *nbox32 = nullptr;  // [(nt-1)*8]: lo xyz, 0, hi xyz, 0 (two 16-byte loads per node)
    double *nbox64 = nullptr; // [(nt-1)*6]
    int *flags = nullptr;     // [nt-1] refit arrival counters
    int *rank = nullptr;      // [nt] position of each triangle in the reference tree's leaf order
    const unsigned int *absMax = nullptr; // [3] per axis: largest |box coordinate|, rounded up to FP32 (bits)
    // the reference tree's nodes: {first leaf position, member count, left child id (the right child is
    // left + 1), -1 for a leaf}; node 0 is the root. Valid with rank.
    int4 *tnode = nullptr;
    int tnodeCount = 0;       // records the node table holds
    unsigned long long *levelStamps = nullptr; // [96] diagnostic: device time per large-node level (3 each)
    bool rankValid = false;
    // [nt*3] for edge k of triangle i (t[k] -> t[k+1]): the first triangle in index order holding the reverse
    // edge, -1 for none. Depends on the triangles only, so a vertex update keeps it.
    int *adj = nullptr;
    int *adjDup = nullptr;    // [1] directed edges held by more than one triangle (0: every edge once)
    int root = 0;             // 0, or ~0 when nt == 1
};

struct sb_mesh_impl;
} // namespace sbg

struct sb_mesh {
    sbg::MeshDev d;
    sbg::DevBuf buf;
    sbg::DevBuf tmp;               // LBVH build temporaries
    sbg::DevBuf rankTmp;           // reference leaf-order temporaries (built concurrently with the LBVH)
    cudaStream_t aux = nullptr;    // second stream of the preparation, created on first use
    cudaEvent_t auxFork = nullptr, auxJoin = nullptr;
    cudaEvent_t readyEv = nullptr; // recorded after the last preparation's work on its own stream
    bool prepared = false;
    bool adjValid = false;         // adj / adjDup computed for the current triangles
    int *rankCheck = nullptr;      // pinned: the leaf-order build's counters, read once its stream is done
    bool rankPending = false;      // rankCheck not yet read (build_reference_rank without waiting)
    bool ownsInput = true;
    cudaStream_t stream = nullptr;
    // preparation stream for callers that pass no stream: a preparation on the legacy default stream would
    // serialise the builds of two meshes; this one forks from it instead (created on first use)
    cudaStream_t own = nullptr;
    cudaEvent_t ownFork = nullptr;
    std::vector<double> hostV;    // only for host-created meshes (kept for re-preparation)
    std::vector<uint32_t> hostT;
};

namespace sbg {
// sb_prepare.cu
// With waitRank false the reference leaf order may still be running on m->aux when this returns: the caller
// orders later work after m->auxJoin and calls reference_rank_result after a synchronisation past it.
sb_status prepare_mesh(sb_mesh *m, int order_mode, cudaStream_t s, bool waitRank = true);
// orders work issued next on s after everything a previous preparation of m issued (its LBVH build on the
// stream it was prepared on, and a leaf-order build still pending on the mesh's second stream); no host wait
sb_status mesh_order_after(sb_mesh *m, cudaStream_t s);
// both meshes of a boolean, each on its own stream, neither joining its leaf order; issued in the order that
// starts the two leaf orders (the longer path) first
sb_status prepare_meshes(sb_mesh *a, cudaStream_t sa, sb_mesh *b, cudaStream_t sb, int order_mode);
// sb_refrank.cu: position of each triangle in the reference tree's leaf order
sb_status build_reference_rank(sb_mesh *m, cudaStream_t s, bool wait);
sb_status reference_rank_result(sb_mesh *m);
int *pinned_slot_acquire();        // 16 ints of pinned host memory (null when none can be allocated)
void pinned_slot_release(int *p);
constexpr size_t kMailBytes = 1024; // a boolean's pinned mailbox for small device-to-host reads
char *pinned_mail_acquire();
void pinned_mail_release(char *p);
} // namespace sbg
