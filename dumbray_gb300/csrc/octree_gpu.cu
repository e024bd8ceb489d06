// octree_gpu.cu - the octree build on the GPU, bit-identical to the host builder (and so to the
// reference's Octree::build, Octree.impl.cuh:114-129, 339-533).
//
// Level by level, like the host builder; per level the GPU runs
//   (1) owner of every reference (binary search over the level's reference ranges),
//   (2) the clipped centre of every reference of a splittable node (parallel over references),
//   (3) the split point of every splittable node: the float sum of its references' centres in list
//       order (a warp per node loads, every lane adds in list order: the order of a float sum is part
//       of the result) and its octants,
//   (4) the octant overlap mask of every reference (parallel),
//   (5) per node the octant occupancy and the split decision (a warp per node; integer sums),
//   (6) the clipped bounds of every reference of a leaf (parallel) and each leaf's box: min / max in
//       list order from the node box, then the padded shrink (a warp per leaf),
//   (7) the children's reference lists: for every split node its references copied to the lists of
//       the octants they overlap, in list order (a warp per node: ballots and prefix counts).
// The host keeps the level bookkeeping (which nodes split, where children and leaf lists go), which
// is the host builder's own step 6, and the final bottom-up box reduce.  All geometry comes from
// octree_geom.h; nvcc compiles it with -fmad=false and IEEE division / square root, the host builder
// with -ffp-contract=off, so both perform the same single-precision operations.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "octree_build.h"
#include "octree_geom.h"

namespace drb {
namespace {

using namespace geom;

const float kBoxEpsGpu = 0.000005f * 256.0f;   // OCTREE_AABB_EPSILON (Octree.impl.cuh:3-5)

__device__ __forceinline__ T3 load_tri(const float *xyz, int id) {
    const float *p = xyz + 9 * (size_t)id;
    return T3{mk(p[0], p[1], p[2]), mk(p[3], p[4], p[5]), mk(p[6], p[7], p[8])};
}
__device__ __forceinline__ Bx load_box(const float *b, int k) {
    const float *p = b + 6 * (size_t)k;
    return Bx{mk(p[0], p[1], p[2]), mk(p[3], p[4], p[5])};
}
__device__ __forceinline__ void store_box(float *b, int k, const Bx &x) {
    float *p = b + 6 * (size_t)k;
    p[0] = x.lo.x; p[1] = x.lo.y; p[2] = x.lo.z;
    p[3] = x.hi.x; p[4] = x.hi.y; p[5] = x.hi.z;
}
__device__ __forceinline__ bool splittable(const int *off, int k, int depth, int max_depth, int split_n) {
    return depth < max_depth && (off[k + 1] - off[k]) >= split_n;
}

__global__ void k_owner(const int *off, int nl, int nr, int *owner) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nr) return;
    int lo = 0, hi = nl - 1;   // last node with off[k] <= r (empty nodes share offsets; take the last)
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= r) lo = mid;
        else hi = mid - 1;
    }
    owner[r] = lo;
}

__global__ void k_centres(const float *xyz, const int *refs, const int *owner, const int *off, const float *box, int nr,
                          int depth, int max_depth, int split_n, float *centre) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nr) return;
    const int k = owner[r];
    if (!splittable(off, k, depth, max_depth, split_n)) return;
    Pieces l, x, y;
    const P3 c = clipped_centre(load_box(box, k), load_tri(xyz, refs[r]), l, x, y);
    centre[3 * (size_t)r] = c.x;
    centre[3 * (size_t)r + 1] = c.y;
    centre[3 * (size_t)r + 2] = c.z;
}

// One warp per node: the lanes load 32 centres at a time and every lane adds them in list order
// (broadcast one by one), so the float sum has the host builder's order.
__global__ void k_split_points(const float *centre, const int *off, const float *box, int nl, int depth, int max_depth,
                               int split_n, float E, float *sub) {
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (k >= nl || !splittable(off, k, depth, max_depth, split_n)) return;
    const int rb = off[k], re = off[k + 1];
    P3 c = mk(0, 0, 0);
    for (int base = rb; base < re; base += 32) {
        const int r = base + lane;
        float x = 0.0f, y = 0.0f, z = 0.0f;
        if (r < re) {
            x = centre[3 * (size_t)r];
            y = centre[3 * (size_t)r + 1];
            z = centre[3 * (size_t)r + 2];
        }
        const int m = min(32, re - base);
        for (int j = 0; j < m; j++)
            c = add(c, mk(__shfl_sync(0xFFFFFFFFu, x, j), __shfl_sync(0xFFFFFFFFu, y, j), __shfl_sync(0xFFFFFFFFu, z, j)));
    }
    if (lane != 0) return;
    c = divs(c, (float)(re - rb));
    Bx o[8];
    octants(load_box(box, k), c, o, E);
    for (int i = 0; i < 8; i++) store_box(sub, 8 * k + i, o[i]);
}

__global__ void k_masks(const float *xyz, const int *refs, const int *owner, const int *off, const float *sub, int nr, int depth,
                        int max_depth, int split_n, unsigned char *mask) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nr) return;
    const int k = owner[r];
    if (!splittable(off, k, depth, max_depth, split_n)) {
        mask[r] = 0;
        return;
    }
    const T3 t = load_tri(xyz, refs[r]);
    unsigned m = 0;
    for (int i = 0; i < 8; i++)
        if (overlaps(load_box(sub, 8 * k + i), t)) m |= 1u << i;
    mask[r] = (unsigned char)m;
}

// splittingMakesSence (Octree.impl.cuh:437-475): one warp per node.
__global__ void k_decide(const unsigned char *mask, const int *off, int nl, int depth, int max_depth, int split_n, int *occ,
                         int *does_split) {
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (k >= nl) return;
    const bool can = splittable(off, k, depth, max_depth, split_n);
    int c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (can)
        for (int r = off[k] + lane; r < off[k + 1]; r += 32) {
            const unsigned m = mask[r];
            for (int i = 0; i < 8; i++) c[i] += (m >> i) & 1u;
        }
    for (int i = 0; i < 8; i++)
        for (int s = 16; s > 0; s >>= 1) c[i] += __shfl_xor_sync(0xFFFFFFFFu, c[i], s);
    if (lane != 0) return;
    bool ok = false;
    if (can) {
        const int cnt = off[k + 1] - off[k];
        int full = 0;
        float load = 0.0f;
        for (int i = 0; i < 8; i++) {
            if (c[i] >= cnt) full++;
            load += ((float)c[i]) / ((float)cnt);
        }
        ok = (full < 1) && (load < fminf(((float)cnt) / ((float)split_n), 6.0f));
    }
    does_split[k] = ok ? 1 : 0;
    for (int i = 0; i < 8; i++) occ[8 * k + i] = c[i];
}

__global__ void k_leaf_bounds(const float *xyz, const int *refs, const int *owner, const float *box, const int *does_split,
                              int nr, float *bounds) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nr) return;
    const int k = owner[r];
    if (does_split[k]) return;
    Pieces l, x, y;
    store_box(bounds, r, clipped_bounds(load_box(box, k), load_tri(xyz, refs[r]), l, x, y));
}

// reduceNode(index, true) of a leaf: min / max over the clipped bounds in list order (broadcast
// from the warp's loads), then shrink.  One warp per leaf.
__global__ void k_leaf_boxes(const float *bounds, const int *off, const float *box, const int *does_split, int nl, float E,
                             float *lbox) {
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (k >= nl || does_split[k]) return;
    const Bx b = load_box(box, k);
    P3 lo = b.hi, hi = b.lo;
    const int rb = off[k], re = off[k + 1];
    for (int base = rb; base < re; base += 32) {
        Bx ob = b;
        if (base + lane < re) ob = load_box(bounds, base + lane);
        const int m = min(32, re - base);
        for (int j = 0; j < m; j++) {
            const float l0 = __shfl_sync(0xFFFFFFFFu, ob.lo.x, j), l1 = __shfl_sync(0xFFFFFFFFu, ob.lo.y, j),
                        l2 = __shfl_sync(0xFFFFFFFFu, ob.lo.z, j);
            const float h0 = __shfl_sync(0xFFFFFFFFu, ob.hi.x, j), h1 = __shfl_sync(0xFFFFFFFFu, ob.hi.y, j),
                        h2 = __shfl_sync(0xFFFFFFFFu, ob.hi.z, j);
            lo = mk(fmin_(lo.x, l0), fmin_(lo.y, l1), fmin_(lo.z, l2));
            hi = mk(fmax_(hi.x, h0), fmax_(hi.y, h1), fmax_(hi.z, h2));
        }
    }
    if (lane == 0) store_box(lbox, k, shrink(b, lo, hi, E));
}

// Children's reference lists (Octree.impl.cuh:392-404): one thread per split node.
__global__ void k_scatter(const int *refs, const unsigned char *mask, const int *off, const int *first_child, const int *next_off,
                          int nl, int *next_refs) {
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (k >= nl || first_child[k] < 0) return;
    const unsigned lt = (1u << lane) - 1u;
    int w[8];
    for (int i = 0; i < 8; i++) w[i] = next_off[first_child[k] + i];
    // chunks of 32 references in list order; within a chunk, a lane's position among the chunk's
    // references overlapping octant i is the count of lower lanes that also do
    for (int base = off[k]; base < off[k + 1]; base += 32) {
        const int r = base + lane;
        const bool in = r < off[k + 1];
        const unsigned m = in ? mask[r] : 0u;
        const int id = in ? refs[r] : 0;
        for (int i = 0; i < 8; i++) {
            const unsigned bal = __ballot_sync(0xFFFFFFFFu, (m >> i) & 1u);
            if ((m >> i) & 1u) next_refs[w[i] + __popc(bal & lt)] = id;
            w[i] += __popc(bal);
        }
    }
}

inline unsigned blocks(long long n, int t) { return (unsigned)((n + t - 1) / t); }

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { cudaFree(p); }
    void swap(DevBuf &o) {
        std::swap(p, o.p);
        std::swap(bytes, o.bytes);
    }
    template <class T>
    T *get(size_t count) {
        const size_t need = std::max<size_t>(count, 1) * sizeof(T);
        if (need > bytes) {
            cudaFree(p);
            p = nullptr;
            bytes = 0;
            if (cudaMalloc(&p, need) != cudaSuccess) return nullptr;
            bytes = need;
        }
        return (T *)p;
    }
};

}  // namespace

bool build_octree_gpu(const float *xyz, int64_t n, const BuildOptions &opt, FlatOctree &out, std::string &err) {
    out = FlatOctree();
    if (n <= 0) return true;
    if (n >= (int64_t(1) << 31)) {
        err = "too many triangles for the device build";
        return false;
    }
    const int max_depth = opt.max_depth > 0 ? opt.max_depth : 24;
    const int split_n = opt.split_threshold > 0 ? opt.split_threshold : 8;
    float E = opt.box_eps > 0.0f ? opt.box_eps : kBoxEpsGpu;
    if (opt.box_eps < 0.0f) {
        float m = 0.0f;
        for (int64_t i = 0; i < 9 * n; i++) m = std::fmax(m, std::fabs(xyz[i]));
        E = std::fmax(m, 1e-30f) * (1.0f / 262144.0f);
    }
    // root box (push, Octree.impl.cuh:97-111): host, serial like the host builder
    Bx root;
    for (int64_t i = 0; i < n; i++) {
        const float *p = xyz + 9 * i;
        Bx b = tri_box(T3{mk(p[0], p[1], p[2]), mk(p[3], p[4], p[5]), mk(p[6], p[7], p[8])});
        if (i == 0) root = b;
        else {
            P3 bl = sub(b.lo, mk(E, E, E)), bh = add(b.hi, mk(E, E, E));
            root = fixed_box(mk(std::fmin(root.lo.x, bl.x), std::fmin(root.lo.y, bl.y), std::fmin(root.lo.z, bl.z)),
                             mk(std::fmax(root.hi.x, bh.x), std::fmax(root.hi.y, bh.y), std::fmax(root.hi.z, bh.z)));
        }
    }

    DevBuf b_xyz, b_refs, b_next, b_owner, b_centre, b_bounds, b_mask, b_off, b_noff, b_box, b_sub, b_occ, b_split, b_lbox, b_fc;
    float *d_xyz = b_xyz.get<float>(9 * (size_t)n);
    int *d_refs = b_refs.get<int>((size_t)n);
    if (!d_xyz || !d_refs) { err = "device allocation failed"; return false; }
    cudaMemcpy(d_xyz, xyz, 36 * (size_t)n, cudaMemcpyHostToDevice);
    {
        std::vector<int> ids((size_t)n);
        for (int64_t i = 0; i < n; i++) ids[i] = (int)i;
        cudaMemcpy(d_refs, ids.data(), 4 * (size_t)n, cudaMemcpyHostToDevice);
    }

    struct LevelNode {
        Bx box;
        int rb, re;
        int64_t global;
    };
    std::vector<LevelNode> level{{root, 0, (int)n, -1}};
    std::vector<Bx> boxes;
    std::vector<int32_t> child;
    std::vector<int64_t> leaf_lo;
    std::vector<int32_t> leaf_cnt;
    std::vector<int32_t> &leaf_refs = out.leaf_refs;
    Bx root_box = root;
    int32_t root_child = -1;
    int64_t root_leaf_lo = 0;
    int32_t root_leaf_cnt = 0;
    int max_seen = 0;
    std::vector<int> h_off, h_split, h_occ, h_refs, h_fc, h_noff;
    std::vector<float> h_box, h_sub, h_lbox;

    for (int depth = 0; !level.empty(); depth++) {
        max_seen = std::max(max_seen, depth);
        const int nl = (int)level.size();
        const int nr = level.back().re;
        h_off.resize(nl + 1);
        h_box.resize(6 * (size_t)nl);
        for (int k = 0; k < nl; k++) {
            h_off[k] = level[k].rb;
            const Bx &b = level[k].box;
            float *p = &h_box[6 * (size_t)k];
            p[0] = b.lo.x; p[1] = b.lo.y; p[2] = b.lo.z; p[3] = b.hi.x; p[4] = b.hi.y; p[5] = b.hi.z;
        }
        h_off[nl] = nr;
        int *d_off = b_off.get<int>(nl + 1);
        float *d_box = b_box.get<float>(6 * (size_t)nl);
        int *d_owner = b_owner.get<int>(nr);
        float *d_centre = b_centre.get<float>(3 * (size_t)nr);
        float *d_sub = b_sub.get<float>(48 * (size_t)nl);
        unsigned char *d_mask = b_mask.get<unsigned char>(nr);
        int *d_occ = b_occ.get<int>(8 * (size_t)nl);
        int *d_split = b_split.get<int>(nl);
        float *d_bounds = b_bounds.get<float>(6 * (size_t)nr);
        float *d_lbox = b_lbox.get<float>(6 * (size_t)nl);
        if (!d_off || !d_box || !d_owner || !d_centre || !d_sub || !d_mask || !d_occ || !d_split || !d_bounds || !d_lbox) {
            err = "device allocation failed";
            return false;
        }
        cudaMemcpy(d_off, h_off.data(), 4 * (size_t)(nl + 1), cudaMemcpyHostToDevice);
        cudaMemcpy(d_box, h_box.data(), 24 * (size_t)nl, cudaMemcpyHostToDevice);
        if (nr > 0) {
            k_owner<<<blocks(nr, 256), 256>>>(d_off, nl, nr, d_owner);
            k_centres<<<blocks(nr, 128), 128>>>(d_xyz, d_refs, d_owner, d_off, d_box, nr, depth, max_depth, split_n, d_centre);
        }
        k_split_points<<<blocks(32LL * nl, 256), 256>>>(d_centre, d_off, d_box, nl, depth, max_depth, split_n, E, d_sub);
        if (nr > 0) k_masks<<<blocks(nr, 128), 128>>>(d_xyz, d_refs, d_owner, d_off, d_sub, nr, depth, max_depth, split_n, d_mask);
        k_decide<<<blocks(32LL * nl, 256), 256>>>(d_mask, d_off, nl, depth, max_depth, split_n, d_occ, d_split);
        if (nr > 0) k_leaf_bounds<<<blocks(nr, 128), 128>>>(d_xyz, d_refs, d_owner, d_box, d_split, nr, d_bounds);
        k_leaf_boxes<<<blocks(32LL * nl, 256), 256>>>(d_bounds, d_off, d_box, d_split, nl, E, d_lbox);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        if (e != cudaSuccess) {
            err = std::string("device build: ") + cudaGetErrorString(e);
            return false;
        }
        h_split.resize(nl);
        h_occ.resize(8 * (size_t)nl);
        h_sub.resize(48 * (size_t)nl);
        h_lbox.resize(6 * (size_t)nl);
        h_refs.resize(nr);
        cudaMemcpy(h_split.data(), d_split, 4 * (size_t)nl, cudaMemcpyDeviceToHost);
        cudaMemcpy(h_occ.data(), d_occ, 32 * (size_t)nl, cudaMemcpyDeviceToHost);
        cudaMemcpy(h_sub.data(), d_sub, 192 * (size_t)nl, cudaMemcpyDeviceToHost);
        cudaMemcpy(h_lbox.data(), d_lbox, 24 * (size_t)nl, cudaMemcpyDeviceToHost);
        if (nr > 0) cudaMemcpy(h_refs.data(), d_refs, 4 * (size_t)nr, cudaMemcpyDeviceToHost);
        auto hbox = [](const std::vector<float> &v, size_t k) {
            const float *p = &v[6 * k];
            return Bx{mk(p[0], p[1], p[2]), mk(p[3], p[4], p[5])};
        };

        // bookkeeping of the host builder's step 6
        std::vector<LevelNode> next;
        h_fc.assign(nl, -1);
        int64_t next_refs = 0;
        for (int k = 0; k < nl; k++) {
            LevelNode &ln = level[k];
            if (!h_split[k]) {
                const int64_t lo = (int64_t)leaf_refs.size();
                leaf_refs.insert(leaf_refs.end(), h_refs.begin() + ln.rb, h_refs.begin() + ln.re);
                const int32_t cnt = ln.re - ln.rb;
                const Bx lb = hbox(h_lbox, k);
                if (ln.global < 0) { root_box = lb; root_leaf_lo = lo; root_leaf_cnt = cnt; }
                else { boxes[ln.global] = lb; leaf_lo[ln.global] = lo; leaf_cnt[ln.global] = cnt; }
                continue;
            }
            const int64_t first = (int64_t)boxes.size();
            if (ln.global < 0) root_child = (int32_t)first;
            else child[ln.global] = (int32_t)first;
            h_fc[k] = (int)next.size();
            for (int i = 0; i < 8; i++) {
                const Bx sb = hbox(h_sub, 8 * (size_t)k + i);
                boxes.push_back(sb);
                child.push_back(-1);
                leaf_lo.push_back(0);
                leaf_cnt.push_back(0);
                LevelNode c;
                c.box = sb;
                c.rb = (int)next_refs;
                next_refs += h_occ[8 * (size_t)k + i];
                c.re = (int)next_refs;
                c.global = first + i;
                next.push_back(c);
            }
        }
        if (next_refs >= (int64_t(1) << 31)) {
            err = "too many references in one level for the device build";
            return false;
        }
        if (!next.empty()) {
            const int nn = (int)next.size();
            h_noff.resize(nn + 1);
            for (int j = 0; j < nn; j++) h_noff[j] = next[j].rb;
            h_noff[nn] = (int)next_refs;
            int *d_fc = b_fc.get<int>(nl);
            int *d_noff = b_noff.get<int>(nn + 1);
            int *d_next = b_next.get<int>((size_t)next_refs);
            if (!d_fc || !d_noff || !d_next) { err = "device allocation failed"; return false; }
            cudaMemcpy(d_fc, h_fc.data(), 4 * (size_t)nl, cudaMemcpyHostToDevice);
            cudaMemcpy(d_noff, h_noff.data(), 4 * (size_t)(nn + 1), cudaMemcpyHostToDevice);
            k_scatter<<<blocks(32LL * nl, 256), 256>>>(d_refs, d_mask, d_off, d_fc, d_noff, nl, d_next);
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaDeviceSynchronize();
            if (e != cudaSuccess) {
                err = std::string("device build: ") + cudaGetErrorString(e);
                return false;
            }
            b_refs.swap(b_next);
            d_refs = (int *)b_refs.p;
        }
        level.swap(next);
    }

    // bottom-up reduce of inner nodes, deeper first (reduceNode(0, false)), as the host builder
    const int64_t nn = (int64_t)boxes.size();
    for (int64_t i = nn - 1; i >= 0; i--) {
        if (child[i] < 0) continue;
        P3 lo = boxes[i].hi, hi = boxes[i].lo;
        for (int c = 0; c < 8; c++) {
            const Bx &cb = boxes[child[i] + c];
            lo = mk(std::fmin(lo.x, cb.lo.x), std::fmin(lo.y, cb.lo.y), std::fmin(lo.z, cb.lo.z));
            hi = mk(std::fmax(hi.x, cb.hi.x), std::fmax(hi.y, cb.hi.y), std::fmax(hi.z, cb.hi.z));
        }
        boxes[i] = shrink(boxes[i], lo, hi, E);
    }
    if (root_child >= 0) {
        P3 lo = root_box.hi, hi = root_box.lo;
        for (int c = 0; c < 8; c++) {
            const Bx &cb = boxes[root_child + c];
            lo = mk(std::fmin(lo.x, cb.lo.x), std::fmin(lo.y, cb.lo.y), std::fmin(lo.z, cb.lo.z));
            hi = mk(std::fmax(hi.x, cb.hi.x), std::fmax(hi.y, cb.hi.y), std::fmax(hi.z, cb.hi.z));
        }
        root_box = shrink(root_box, lo, hi, E);
    }
    out.node_count = nn;
    out.node_lo.resize(3 * nn);
    out.node_hi.resize(3 * nn);
    out.node_child = std::move(child);
    out.node_leaf_first.resize(nn);
    out.node_leaf_count = std::move(leaf_cnt);
    for (int64_t i = 0; i < nn; i++) {
        out.node_lo[3 * i] = boxes[i].lo.x; out.node_lo[3 * i + 1] = boxes[i].lo.y; out.node_lo[3 * i + 2] = boxes[i].lo.z;
        out.node_hi[3 * i] = boxes[i].hi.x; out.node_hi[3 * i + 1] = boxes[i].hi.y; out.node_hi[3 * i + 2] = boxes[i].hi.z;
        out.node_leaf_first[i] = leaf_lo[i];
    }
    out.root_lo[0] = root_box.lo.x; out.root_lo[1] = root_box.lo.y; out.root_lo[2] = root_box.lo.z;
    out.root_hi[0] = root_box.hi.x; out.root_hi[1] = root_box.hi.y; out.root_hi[2] = root_box.hi.z;
    out.root_child = root_child;
    out.root_leaf_first = root_leaf_lo;
    out.root_leaf_count = root_leaf_cnt;
    out.depth = max_seen;
    return true;
}

}  // namespace drb
