// bvh_build.cu -- device binned-SAH build, collapsed to 8-wide quantised nodes.
//
// Replaces BVH8::Create / SplitSAH (src/s3d_bvh8.cpp:254-342,401-479), which splits a
// range three binary levels deep with a 16-bucket SAH on the longest centroid axis and
// recurses on the CPU.  Here:
//   1. a binary tree is built breadth first, one level per pass over all primitives:
//      32 bins on each of the three centroid axes, cost = ntrav*SA(node) +
//      nL*SA(L) + nR*SA(R) against count*SA(node) for a leaf (the reference's cost form,
//      src/s3d_bvh8.cpp:300-317; ntrav is 0.3 by default instead of its 1, since small
//      leaves trace fastest here), leaves of at most 3 triangles;
//      ranges larger than kSmall are binned by all threads with block-aggregated atomics,
//      smaller ones by one warp in shared memory;
//   2. the binary tree is collapsed into 8-wide nodes: dynamic programming over the binary
//      tree picks the SAH-cheapest choice of wide nodes, leaves (subtrees of up to three
//      triangles) and opened nodes; the wide nodes are then written top down;
//   3. child boxes are quantised to 8 bits per plane against a per-node power-of-two
//      grid, rounding outward, so every quantised box contains the exact one.
#include <cfloat>
#include <cmath>

#include <atomic>
#include <vector>

#include "internal.h"

namespace salty {
namespace {

constexpr int kBins = 32;
// SAH weights of the collapse: one 8-wide node visit against one triangle test.  Measured
// on the traversal microbenchmark and the 1080p heightfield (GB300): any triangle weight
// from 1 to 2.6 node visits gives the same speed within noise, lighter ones put more
// triangles in each leaf and lose 3-10 %.
constexpr float kCollapseNodeCost = 1.0f;
constexpr float kCollapseTriCost = 2.0f;
constexpr int kSmall = 256;
constexpr int kBinWords = 3 * kBins * 7;  // count + lo[3] + hi[3] per bin per axis

__device__ __forceinline__ int f2o(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float o2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

struct Task {
    int node, first, count, bin_slot;
    int cmin[3], cmax[3];          // ordered-int centroid bounds
    int mode, axis, split, nleft;  // mode: 0 open, 1 leaf, 2 bin split, 3 median split
    int child_task, cursor[2], pad;
};
static_assert(sizeof(Task) == 72, "task");

struct Counters {
    int nodes;        // binary nodes allocated
    int next_tasks;   // tasks of the next level
    int next_large;   // bin slots of the next level
    int depth;
    int n8;           // BVH8 nodes allocated
    int ntris;        // leaf triangles written
    int next_work;    // collapse work items of the next level
    int error;        // set when a partition slot falls outside its range
    double sah;       // accumulated SAH numerator
    int rootbox[6];   // ordered-int bounds of all primitive boxes
    int rootcen[6];   // ordered-int bounds of all centroids
};

__device__ __forceinline__ int bin_of(float c, float cmin, float cmax, int B) {
    float ext = cmax - cmin;
    if (!(ext > 0.0f)) return 0;
    float k = (float)B / ext;
    int b = (int)((c - cmin) * k);
    return min(max(b, 0), B - 1);
}

__device__ __forceinline__ float area(float dx, float dy, float dz) {
    dx = fmaxf(dx, 0.0f); dy = fmaxf(dy, 0.0f); dz = fmaxf(dz, 0.0f);
    return 2.0f * (dx * dy + dx * dz + dy * dz);
}

// ---------------------------------------------------------------- setup
__global__ void k_prim_setup(const float* __restrict__ pos, int n, float4* __restrict__ lo4,
                             float4* __restrict__ hi4, float4* __restrict__ cen4, int* __restrict__ prim,
                             int* __restrict__ pos_task, Counters* ctr) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    float c[3] = {0, 0, 0};
    bool valid = i < n;
    if (valid) {
        const float* p = pos + (size_t)i * 9;
        for (int a = 0; a < 3; ++a) {
            lo[a] = fminf(p[a], fminf(p[3 + a], p[6 + a]));
            hi[a] = fmaxf(p[a], fmaxf(p[3 + a], p[6 + a]));
            c[a] = (lo[a] + hi[a]) * 0.5f;  // BoundingBox::center (include/s3d_math.h:2178-2183)
        }
        lo4[i] = make_float4(lo[0], lo[1], lo[2], 0.0f);
        hi4[i] = make_float4(hi[0], hi[1], hi[2], 0.0f);
        cen4[i] = make_float4(c[0], c[1], c[2], 0.0f);
        prim[i] = i;
        pos_task[i] = 0;
    }
    // warp-reduce bounds, one atomic per warp
    for (int a = 0; a < 3; ++a) {
        int vlo = f2o(lo[a]), vhi = f2o(hi[a]);
        int clo = valid ? f2o(c[a]) : f2o(FLT_MAX), chi = valid ? f2o(c[a]) : f2o(-FLT_MAX);
        vlo = __reduce_min_sync(0xffffffffu, vlo);
        vhi = __reduce_max_sync(0xffffffffu, vhi);
        clo = __reduce_min_sync(0xffffffffu, clo);
        chi = __reduce_max_sync(0xffffffffu, chi);
        if ((threadIdx.x & 31) == 0) {
            atomicMin(&ctr->rootbox[a], vlo);
            atomicMax(&ctr->rootbox[3 + a], vhi);
            atomicMin(&ctr->rootcen[a], clo);
            atomicMax(&ctr->rootcen[3 + a], chi);
        }
    }
}

__global__ void k_root_init(Counters* ctr, Task* tasks, BNode* nodes, int n, int bins_small) {
    Task t;
    t.node = 0; t.first = 0; t.count = n;
    t.bin_slot = (n > kSmall) ? 0 : -1;
    for (int a = 0; a < 3; ++a) { t.cmin[a] = ctr->rootcen[a]; t.cmax[a] = ctr->rootcen[3 + a]; }
    t.mode = 0; t.axis = 0; t.split = 0; t.nleft = 0; t.child_task = 0;
    t.cursor[0] = t.cursor[1] = 0; t.pad = 0;
    tasks[0] = t;
    BNode r;
    for (int a = 0; a < 3; ++a) { r.lo[a] = o2f(ctr->rootbox[a]); r.hi[a] = o2f(ctr->rootbox[3 + a]); }
    r.a = 0; r.count = 0;
    nodes[0] = r;
    ctr->nodes = 1;
    ctr->next_large = (n > kSmall) ? 1 : 0;
    (void)bins_small;
}

// ---------------------------------------------------------------- binning (large tasks)
__global__ void k_clear_bins(int* bins, int nslots) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int total = nslots * kBinWords;
    if (i >= total) return;
    int w = i % 7;
    bins[i] = (w == 0) ? 0 : (w <= 3 ? f2o(FLT_MAX) : f2o(-FLT_MAX));
}

__global__ void k_bin(int n, const int* __restrict__ pos_task, const int* __restrict__ prim,
                      const float4* __restrict__ cen4, const float4* __restrict__ lo4,
                      const float4* __restrict__ hi4, const Task* __restrict__ tasks, int* bins, int B) {
    __shared__ int sb[kBinWords];
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    int t = (p < n) ? pos_task[p] : -1;
    int slot = -1;
    Task tk;
    if (t >= 0) {
        tk = tasks[t];
        slot = tk.bin_slot;
        if (tk.count <= kSmall) slot = -1;
    }
    int first_slot = __shfl_sync(0xffffffffu, slot, 0);
    __shared__ int s_slot0;
    if (threadIdx.x == 0) s_slot0 = slot;
    __syncthreads();
    bool uniform = __syncthreads_and(slot == s_slot0 && slot >= 0);
    (void)first_slot;
    float c[3], lo[3], hi[3];
    if (slot >= 0) {
        int q = prim[p];
        float4 cc = cen4[q], l = lo4[q], h = hi4[q];
        c[0] = cc.x; c[1] = cc.y; c[2] = cc.z;
        lo[0] = l.x; lo[1] = l.y; lo[2] = l.z;
        hi[0] = h.x; hi[1] = h.y; hi[2] = h.z;
    }
    if (uniform) {
        for (int i = threadIdx.x; i < kBinWords; i += blockDim.x) {
            int w = i % 7;
            sb[i] = (w == 0) ? 0 : (w <= 3 ? f2o(FLT_MAX) : f2o(-FLT_MAX));
        }
        __syncthreads();
        for (int a = 0; a < 3; ++a) {
            int b = bin_of(c[a], o2f(tk.cmin[a]), o2f(tk.cmax[a]), B);
            int* s = sb + (a * kBins + b) * 7;
            atomicAdd(s, 1);
            for (int k = 0; k < 3; ++k) {
                atomicMin(s + 1 + k, f2o(lo[k]));
                atomicMax(s + 4 + k, f2o(hi[k]));
            }
        }
        __syncthreads();
        int* g = bins + (size_t)slot * kBinWords;
        for (int i = threadIdx.x; i < 3 * kBins; i += blockDim.x) {
            int* s = sb + i * 7;
            if (s[0] == 0) continue;
            atomicAdd(g + i * 7, s[0]);
            for (int k = 0; k < 3; ++k) {
                atomicMin(g + i * 7 + 1 + k, s[1 + k]);
                atomicMax(g + i * 7 + 4 + k, s[4 + k]);
            }
        }
    } else if (slot >= 0) {
        int* g = bins + (size_t)slot * kBinWords;
        for (int a = 0; a < 3; ++a) {
            int b = bin_of(c[a], o2f(tk.cmin[a]), o2f(tk.cmax[a]), B);
            int* s = g + (a * kBins + b) * 7;
            atomicAdd(s, 1);
            for (int k = 0; k < 3; ++k) {
                atomicMin(s + 1 + k, f2o(lo[k]));
                atomicMax(s + 4 + k, f2o(hi[k]));
            }
        }
    }
}

// ---------------------------------------------------------------- split decision
struct BuildParams {
    int B;
    int max_leaf;
    float trav_cost;
};

constexpr int kSplitWarps = 4;

__global__ void __launch_bounds__(kSplitWarps * 32)
k_split(Task* tasks, int ntasks, const int* bins, BNode* nodes, const int* __restrict__ prim,
        const float4* __restrict__ cen4, const float4* __restrict__ lo4, const float4* __restrict__ hi4,
        BuildParams prm, Counters* ctr, Task* tasks_next, int level) {
    __shared__ int sb[kSplitWarps][kBinWords];
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int t = blockIdx.x * kSplitWarps + warp;
    if (t >= ntasks) return;
    Task tk = tasks[t];
    const int B = prm.B;
    const int* g;
    if (tk.count > kSmall) {
        g = bins + (size_t)tk.bin_slot * kBinWords;
    } else {
        int* s = sb[warp];
        for (int i = lane; i < kBinWords; i += 32) {
            int w = i % 7;
            s[i] = (w == 0) ? 0 : (w <= 3 ? f2o(FLT_MAX) : f2o(-FLT_MAX));
        }
        __syncwarp();
        if (tk.count > 1) {
            for (int i = lane; i < tk.count; i += 32) {
                int q = prim[tk.first + i];
                float4 cc = cen4[q], l = lo4[q], h = hi4[q];
                float c[3] = {cc.x, cc.y, cc.z}, lo[3] = {l.x, l.y, l.z}, hi[3] = {h.x, h.y, h.z};
                for (int a = 0; a < 3; ++a) {
                    int b = bin_of(c[a], o2f(tk.cmin[a]), o2f(tk.cmax[a]), B);
                    int* e = s + (a * kBins + b) * 7;
                    atomicAdd(e, 1);
                    for (int k = 0; k < 3; ++k) {
                        atomicMin(e + 1 + k, f2o(lo[k]));
                        atomicMax(e + 4 + k, f2o(hi[k]));
                    }
                }
            }
        }
        __syncwarp();
        g = s;
    }

    BNode nd = nodes[tk.node];
    float node_sa = area(nd.hi[0] - nd.lo[0], nd.hi[1] - nd.lo[1], nd.hi[2] - nd.lo[2]);

    float best_cost = INFINITY;
    int best_axis = -1, best_bin = -1, best_nl = 0;
    float bl_lo[3], bl_hi[3], br_lo[3], br_hi[3];
    for (int a = 0; a < 3; ++a) {
        int cnt = 0;
        float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        if (lane < B) {
            const int* e = g + (a * kBins + lane) * 7;
            cnt = e[0];
            for (int k = 0; k < 3; ++k) { lo[k] = o2f(e[1 + k]); hi[k] = o2f(e[4 + k]); }
        }
        // inclusive prefix (left) and suffix (right)
        int lc = cnt, rc = cnt;
        float llo[3], lhi[3], rlo[3], rhi[3];
        for (int k = 0; k < 3; ++k) { llo[k] = rlo[k] = lo[k]; lhi[k] = rhi[k] = hi[k]; }
        for (int off = 1; off < 32; off <<= 1) {
            int v = __shfl_up_sync(0xffffffffu, lc, off);
            int w = __shfl_down_sync(0xffffffffu, rc, off);
            if (lane >= off) lc += v;
            if (lane + off < 32) rc += w;
            for (int k = 0; k < 3; ++k) {
                float a1 = __shfl_up_sync(0xffffffffu, llo[k], off);
                float a2 = __shfl_up_sync(0xffffffffu, lhi[k], off);
                float b1 = __shfl_down_sync(0xffffffffu, rlo[k], off);
                float b2 = __shfl_down_sync(0xffffffffu, rhi[k], off);
                if (lane >= off) { llo[k] = fminf(llo[k], a1); lhi[k] = fmaxf(lhi[k], a2); }
                if (lane + off < 32) { rlo[k] = fminf(rlo[k], b1); rhi[k] = fmaxf(rhi[k], b2); }
            }
        }
        // split after bin `lane`: left = prefix[lane], right = suffix[lane + 1]
        int nr = __shfl_down_sync(0xffffffffu, rc, 1);
        float srlo[3], srhi[3];
        for (int k = 0; k < 3; ++k) {
            srlo[k] = __shfl_down_sync(0xffffffffu, rlo[k], 1);
            srhi[k] = __shfl_down_sync(0xffffffffu, rhi[k], 1);
        }
        bool ok = (lane < B - 1) && lc > 0 && nr > 0;
        float cost = ok ? (float)lc * area(lhi[0] - llo[0], lhi[1] - llo[1], lhi[2] - llo[2]) +
                              (float)nr * area(srhi[0] - srlo[0], srhi[1] - srlo[1], srhi[2] - srlo[2])
                        : INFINITY;
        // arg-min over lanes (ties -> lower lane)
        float mc = cost;
        int ml = lane;
        for (int off = 16; off > 0; off >>= 1) {
            float oc = __shfl_xor_sync(0xffffffffu, mc, off);
            int ol = __shfl_xor_sync(0xffffffffu, ml, off);
            if (oc < mc || (oc == mc && ol < ml)) { mc = oc; ml = ol; }
        }
        if (mc < best_cost) {
            best_cost = mc;
            best_axis = a;
            best_bin = ml;
            best_nl = __shfl_sync(0xffffffffu, lc, ml);
            for (int k = 0; k < 3; ++k) {
                bl_lo[k] = __shfl_sync(0xffffffffu, llo[k], ml);
                bl_hi[k] = __shfl_sync(0xffffffffu, lhi[k], ml);
                br_lo[k] = __shfl_sync(0xffffffffu, srlo[k], ml);
                br_hi[k] = __shfl_sync(0xffffffffu, srhi[k], ml);
            }
        }
    }
    if (lane != 0) return;

    int mode;
    float leaf_cost = (float)tk.count * node_sa;
    float split_cost = prm.trav_cost * node_sa + best_cost;
    if (tk.count <= 1) mode = 1;
    else if (tk.count <= prm.max_leaf && leaf_cost <= split_cost) mode = 1;
    else if (best_axis >= 0 && best_cost < INFINITY) mode = 2;
    else if (tk.count <= prm.max_leaf) mode = 1;
    else mode = 3;

    Task& out = tasks[t];
    out.mode = mode;
    atomicMax(&ctr->depth, level + 1);
    if (mode == 1) {
        nodes[tk.node].a = tk.first;
        nodes[tk.node].count = tk.count;
        return;
    }
    int nl = (mode == 2) ? best_nl : tk.count / 2;
    if (mode == 3) {
        for (int k = 0; k < 3; ++k) {
            bl_lo[k] = br_lo[k] = nd.lo[k];
            bl_hi[k] = br_hi[k] = nd.hi[k];
        }
    }
    out.axis = best_axis;
    out.split = best_bin;
    out.nleft = nl;
    int cid = atomicAdd(&ctr->nodes, 2);
    int t0 = atomicAdd(&ctr->next_tasks, 2);
    out.child_task = t0;
    nodes[tk.node].a = cid;
    nodes[tk.node].count = 0;
    BNode L, R;
    for (int k = 0; k < 3; ++k) { L.lo[k] = bl_lo[k]; L.hi[k] = bl_hi[k]; R.lo[k] = br_lo[k]; R.hi[k] = br_hi[k]; }
    L.a = R.a = 0; L.count = R.count = 0;
    nodes[cid] = L;
    nodes[cid + 1] = R;
    for (int s = 0; s < 2; ++s) {
        Task c;
        c.node = cid + s;
        c.first = tk.first + (s ? nl : 0);
        c.count = s ? tk.count - nl : nl;
        c.bin_slot = (c.count > kSmall) ? atomicAdd(&ctr->next_large, 1) : -1;
        for (int k = 0; k < 3; ++k) { c.cmin[k] = f2o(FLT_MAX); c.cmax[k] = f2o(-FLT_MAX); }
        c.mode = 0; c.axis = 0; c.split = 0; c.nleft = 0; c.child_task = 0;
        c.cursor[0] = c.cursor[1] = 0; c.pad = 0;
        tasks_next[t0 + s] = c;
    }
}

// ---------------------------------------------------------------- partition
__global__ void k_partition(int n, const int* __restrict__ pos_task, const int* __restrict__ prim,
                            const float4* __restrict__ cen4, Task* tasks, Task* tasks_next,
                            int* __restrict__ prim_next, int* __restrict__ pos_task_next, int B,
                            Counters* ctr) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    int lane = threadIdx.x & 31;
    bool inb = p < n;
    int t = inb ? pos_task[p] : -1;
    int q = inb ? prim[p] : 0;
    Task tk;
    bool split = false;
    int side = 0;
    float c[3] = {0, 0, 0};
    if (t >= 0) {
        tk = tasks[t];
        split = (tk.mode == 2 || tk.mode == 3);
    }
    if (inb && !split) {
        prim_next[p] = q;
        pos_task_next[p] = -1;
    }
    if (split) {
        float4 cc = cen4[q];
        c[0] = cc.x; c[1] = cc.y; c[2] = cc.z;
        if (tk.mode == 2) {
            int a = tk.axis;
            side = bin_of(c[a], o2f(tk.cmin[a]), o2f(tk.cmax[a]), B) > tk.split ? 1 : 0;
        } else {
            side = (p - tk.first) >= tk.nleft ? 1 : 0;
        }
    }
    int key = split ? (t * 2 + side) : -(lane + 1);
    unsigned m = __match_any_sync(0xffffffffu, key);
    if (!split) return;
    int leader = __ffs(m) - 1;
    int rank = __popc(m & ((1u << lane) - 1));
    int base = 0;
    if (lane == leader) base = atomicAdd(&tasks[t].cursor[side], __popc(m));
    base = __shfl_sync(m, base, leader);
    int np = tk.first + (side ? tk.nleft : 0) + base + rank;
    int ct = tk.child_task + side;
    const int lo = tk.first + (side ? tk.nleft : 0), hi = side ? tk.first + tk.count : tk.first + tk.nleft;
    if (np < lo || np >= hi) {  // binning and partition disagree: report, never write out of range
        atomicOr(&ctr->error, 1);
        return;
    }
    prim_next[np] = q;
    pos_task_next[np] = ct;
    Task* ch = &tasks_next[ct];
    if (m == 0xffffffffu) {
        for (int a = 0; a < 3; ++a) {
            int vmin = __reduce_min_sync(0xffffffffu, f2o(c[a]));
            int vmax = __reduce_max_sync(0xffffffffu, f2o(c[a]));
            if (lane == 0) {
                atomicMin(&ch->cmin[a], vmin);
                atomicMax(&ch->cmax[a], vmax);
            }
        }
    } else {
        for (int a = 0; a < 3; ++a) {
            atomicMin(&ch->cmin[a], f2o(c[a]));
            atomicMax(&ch->cmax[a], f2o(c[a]));
        }
    }
}

// ---------------------------------------------------------------- collapse + quantise
__device__ __forceinline__ float bnode_area(const BNode& b) {
    return area(b.hi[0] - b.lo[0], b.hi[1] - b.lo[1], b.hi[2] - b.lo[2]);
}

// Per-axis power-of-two grid: the smallest 2^e with 255 * 2^e >= hi - lo.
__device__ int quant_exponent(float lo, float hi) {
    double ext = (double)hi - (double)lo;
    if (!(ext > 0.0)) return -126;
    int e;
    frexp(ext / 255.0, &e);  // ext/255 = m * 2^e, m in [0.5, 1)
    while (255.0 * ldexp(1.0, e) < ext) ++e;
    while (e > -126 && 255.0 * ldexp(1.0, e - 1) >= ext) --e;
    if (e < -126) e = -126;
    if (e > 127) e = 127;
    return e;
}

// ---------------------------------------------------------------- SAH-optimal collapse
// Which binary nodes become 8-wide nodes, which become leaves of the wide tree, and which
// are opened into their parent's child slots is decided by dynamic programming over the
// binary tree (Ylitie, Karras, Laine, "Efficient Incoherent Ray Traversal on GPUs Through
// Compressed Wide BVHs", HPG 2017, section 3.1): for every binary node n and every
// i = 1..7, C(n, i) is the least SAH cost of covering n's subtree with at most i roots, each
// an 8-wide node or a leaf of at most kMaxLeafTris triangles:
//   C(n, 1)  = min(leaf: A(n) p(n) c_tri  if p(n) <= kMaxLeafTris,
//                  node: A(n) c_node + D(n, 8))
//   C(n, i)  = min(C(n, i - 1), D(n, i))                           i = 2..7
//   D(n, j)  = min over k = 1..j-1 of C(left, k) + C(right, j - k)
// with A the surface area and p the triangle count.  Binary leaves can only be leaves.
// The nodes of one binary level are solved together, deepest level first.
struct CollapseDP {
    float c[7];          // C(n, 1..7)
    int first, count;    // the subtree's triangles: prim positions [first, first + count)
    unsigned dec;        // bit 0: C(n, 1) is a leaf; bits 1..6: C(n, i) takes D(n, i), i = 2..7;
                         // bits 8 + 3 (j - 2): the k of D(n, j), j = 2..8
};

__global__ void k_collapse_dp(const BNode* __restrict__ bn, CollapseDP* __restrict__ dp, int begin, int end,
                              float c_node, float c_tri) {
    const int i = begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= end) return;
    const BNode b = bn[i];
    const float A = bnode_area(b);
    CollapseDP r;
    if (b.count > 0) {
        r.first = b.a;
        r.count = b.count;
        const float leaf = A * (float)b.count * c_tri;
        for (int k = 0; k < 7; ++k) r.c[k] = leaf;
        r.dec = 1u;
        dp[i] = r;
        return;
    }
    const CollapseDP L = dp[b.a], R = dp[b.a + 1];
    r.first = min(L.first, R.first);
    r.count = L.count + R.count;
    float D[9];
    unsigned dec = 0;
    for (int j = 2; j <= 8; ++j) {
        float best = INFINITY;
        int bk = 1;
        for (int k = 1; k < j; ++k) {
            const int kr = j - k;
            if (k > 7 || kr > 7) continue;
            const float v = L.c[k - 1] + R.c[kr - 1];
            if (v < best) { best = v; bk = k; }
        }
        D[j] = best;
        dec |= (unsigned)bk << (8 + 3 * (j - 2));
    }
    const float node = A * c_node + D[8];
    const float leaf = r.count <= kMaxLeafTris ? A * (float)r.count * c_tri : INFINITY;
    if (leaf <= node) { r.c[0] = leaf; dec |= 1u; }
    else r.c[0] = node;
    for (int k = 2; k <= 7; ++k) {
        if (D[k] < r.c[k - 2]) { r.c[k - 1] = D[k]; dec |= 1u << (k - 1); }
        else r.c[k - 1] = r.c[k - 2];
    }
    r.dec = dec;
    dp[i] = r;
}

// The children of the 8-wide node made from binary node `bid`: D(bid, 8) unfolded.  Each
// child is a binary node standing for itself (leaf[] tells whether as a leaf of the wide
// tree or as an 8-wide node).  Returns the number of children (1..8).
__device__ int collapse_children(const BNode* __restrict__ bn, const CollapseDP* __restrict__ dp, int bid,
                                 int* set, bool* leaf) {
    int k = 0;
    if (bn[bid].count > 0) {  // a binary leaf at the root: one leaf child
        set[0] = bid;
        leaf[0] = true;
        return 1;
    }
    int sn[16], sj[16], sp = 0;
    sn[sp] = bid; sj[sp] = 8; ++sp;
    bool top = true;
    while (sp > 0) {
        --sp;
        const int m = sn[sp];
        int j = sj[sp];
        const BNode b = bn[m];
        const unsigned dec = dp[m].dec;
        if (!top) {
            if (b.count > 0) { set[k] = m; leaf[k] = true; ++k; continue; }
            while (j > 1 && j <= 7 && !((dec >> (j - 1)) & 1u)) --j;  // C(m, j) = C(m, j - 1)
            if (j == 1) { set[k] = m; leaf[k] = (dec & 1u) != 0; ++k; continue; }
        }
        top = false;
        const int kl = (dec >> (8 + 3 * (j - 2))) & 7u;
        sn[sp] = b.a + 1; sj[sp] = j - kl; ++sp;  // right, visited after left
        sn[sp] = b.a; sj[sp] = kl; ++sp;
    }
    return k;
}

__global__ void k_collapse(const BNode* __restrict__ bn, int nwork, const int2* __restrict__ work,
                           Bvh8Node* __restrict__ out, float4* __restrict__ tris,
                           const int* __restrict__ prim, const float* __restrict__ pos,
                           int2* __restrict__ work_next, Counters* ctr, float root_sa,
                           const CollapseDP* __restrict__ dp) {
    int wi = blockIdx.x * blockDim.x + threadIdx.x;
    if (wi >= nwork) return;
    int bid = work[wi].x, oid = work[wi].y;
    BNode b = bn[bid];
    int set[8];
    bool as_leaf[8];
    const int k = collapse_children(bn, dp, bid, set, as_leaf);
    // slot assignment by octant of the child centre around the node centre
    float cx = (b.lo[0] + b.hi[0]) * 0.5f, cy = (b.lo[1] + b.hi[1]) * 0.5f, cz = (b.lo[2] + b.hi[2]) * 0.5f;
    int slot_child[8];
    for (int s = 0; s < 8; ++s) slot_child[s] = -1;
    // place larger children first so they get their preferred slot
    int order[8];
    float osa[8];
    for (int i = 0; i < k; ++i) { order[i] = i; osa[i] = bnode_area(bn[set[i]]); }
    for (int i = 1; i < k; ++i) {
        int o = order[i]; float s = osa[o]; int j = i - 1;
        while (j >= 0 && osa[order[j]] < s) { order[j + 1] = order[j]; --j; }
        order[j + 1] = o;
    }
    for (int ii = 0; ii < k; ++ii) {
        int i = order[ii];
        BNode c = bn[set[i]];
        int pref = (((c.lo[0] + c.hi[0]) * 0.5f > cx) ? 1 : 0) | (((c.lo[1] + c.hi[1]) * 0.5f > cy) ? 2 : 0) |
                   (((c.lo[2] + c.hi[2]) * 0.5f > cz) ? 4 : 0);
        int bs = -1, bd = 99;
        for (int s = 0; s < 8; ++s) {
            if (slot_child[s] >= 0) continue;
            int d = __popc(s ^ pref);
            if (d < bd) { bd = d; bs = s; }
        }
        slot_child[bs] = i;
    }
    int n_int = 0, n_tri = 0;
    for (int i = 0; i < k; ++i) {
        if (!as_leaf[i]) ++n_int; else n_tri += dp[set[i]].count;
    }
    int child_base = n_int ? atomicAdd(&ctr->n8, n_int) : 0;
    int tri_base = n_tri ? atomicAdd(&ctr->ntris, n_tri) : 0;
    int ex[3];
    for (int a = 0; a < 3; ++a) ex[a] = quant_exponent(b.lo[a], b.hi[a]);
    double sc[3];
    for (int a = 0; a < 3; ++a) sc[a] = ldexp(1.0, ex[a]);
    unsigned char qlo[3][8], qhi[3][8], meta[8];
    unsigned imask = 0;
    int r_int = 0, off = 0;
    double sah = (double)bnode_area(b);
    for (int s = 0; s < 8; ++s) {
        meta[s] = 0;
        int i = slot_child[s];
        if (i < 0) {
            for (int a = 0; a < 3; ++a) { qlo[a][s] = 255; qhi[a][s] = 0; }
            continue;
        }
        BNode c = bn[set[i]];
        for (int a = 0; a < 3; ++a) {
            double lo = floor(((double)c.lo[a] - (double)b.lo[a]) / sc[a]);
            double hi = ceil(((double)c.hi[a] - (double)b.lo[a]) / sc[a]);
            qlo[a][s] = (unsigned char)fmin(fmax(lo, 0.0), 255.0);
            qhi[a][s] = (unsigned char)fmin(fmax(hi, 0.0), 255.0);
        }
        // a leaf child holds the triangles of its whole binary subtree
        c.a = dp[set[i]].first;
        c.count = as_leaf[i] ? dp[set[i]].count : 0;
        if (c.count == 0) {
            imask |= 1u << s;
            meta[s] = (unsigned char)((1u << 5) | (24u + s));  // one hit bit at 24 + slot
            int idx = child_base + r_int++;
            int w = atomicAdd(&ctr->next_work, 1);
            work_next[w] = make_int2(set[i], idx);
        } else {
            // unary triangle count in the top three bits, first triangle in the low five
            meta[s] = (unsigned char)((((1u << c.count) - 1u) << 5) | off);
            for (int j = 0; j < c.count; ++j) {
                int q = prim[c.a + j];
                const float* p = pos + (size_t)q * 9;
                float4* dst = tris + (size_t)(tri_base + off + j) * kTriFloat4;
                dst[0] = make_float4(p[0], p[1], p[2], __int_as_float(q));
                dst[1] = make_float4(p[3], p[4], p[5], 0.0f);
                dst[2] = make_float4(p[6], p[7], p[8], 0.0f);
            }
            off += c.count;
            sah += (double)c.count * (double)bnode_area(c);
        }
    }
    Bvh8Node nd;
    nd.w[0] = make_uint4(__float_as_uint(b.lo[0]), __float_as_uint(b.lo[1]), __float_as_uint(b.lo[2]),
                         (unsigned)(ex[0] + 127) | ((unsigned)(ex[1] + 127) << 8) |
                             ((unsigned)(ex[2] + 127) << 16) | (imask << 24));
    auto pack4 = [](const unsigned char* v) {
        return (unsigned)v[0] | ((unsigned)v[1] << 8) | ((unsigned)v[2] << 16) | ((unsigned)v[3] << 24);
    };
    nd.w[1] = make_uint4((unsigned)child_base, (unsigned)tri_base, pack4(meta), pack4(meta + 4));
    nd.w[2] = make_uint4(pack4(qlo[0]), pack4(qlo[0] + 4), pack4(qlo[1]), pack4(qlo[1] + 4));
    nd.w[3] = make_uint4(pack4(qlo[2]), pack4(qlo[2] + 4), pack4(qhi[0]), pack4(qhi[0] + 4));
    nd.w[4] = make_uint4(pack4(qhi[1]), pack4(qhi[1] + 4), pack4(qhi[2]), pack4(qhi[2] + 4));
    out[oid] = nd;
    atomicAdd(&ctr->sah, sah / (double)root_sa);
}

__global__ void k_init_counters(Counters* c) {
    Counters z;
    memset(&z, 0, sizeof(z));
    for (int a = 0; a < 3; ++a) {
        z.rootbox[a] = f2o(FLT_MAX); z.rootbox[3 + a] = f2o(-FLT_MAX);
        z.rootcen[a] = f2o(FLT_MAX); z.rootcen[3 + a] = f2o(-FLT_MAX);
    }
    *c = z;
}

inline unsigned grid_for(long long n, int block) { return (unsigned)((n + block - 1) / block); }

}  // namespace

salty_status build_bvh(salty_ctx* ctx, salty_scene* sc, const salty_build_opts& opts) {
    if (sc->n_inst > 0) return build_instanced(ctx, sc, opts);
    if (sc->n_sph > 0) return build_with_spheres(ctx, sc, opts);
    if (sc->n_tris <= 0) return ctx->err.fail(SALTY_ERR_INVALID_ARG, "scene has no triangles");
    if (sc->n_tris > (int64_t)0x3fffffff)
        return ctx->err.fail(SALTY_ERR_CAPACITY, "too many triangles (%lld)", (long long)sc->n_tris);
    float box[6];
    return build_bvh_tris(ctx, sc->pos.p, (int)sc->n_tris, opts, sc->bvh, box);
}

salty_status build_bvh_tris(salty_ctx* ctx, const float* d_pos, int n, const salty_build_opts& opts, Bvh& out,
                            float root_box[6]) {
    auto& E = ctx->err;
    if (n <= 0) return E.fail(SALTY_ERR_INVALID_ARG, "no triangles to build a BVH over");
    BuildParams prm;
    prm.B = opts.bins;
    prm.max_leaf = opts.max_leaf;
    prm.trav_cost = opts.trav_cost;
    cudaStream_t st = ctx->stream;

    DevBuf<float4> lo4, hi4, cen4;
    DevBuf<int> prim[2], pos_task[2];
    DevBuf<Task> tasks[2];
    DevBuf<BNode> bnodes;
    DevBuf<int> bins;
    DevBuf<Counters> ctr;
    DevBuf<int2> work[2];
    SALTY_TRY_CUDA(E, lo4.ensure(n));
    SALTY_TRY_CUDA(E, hi4.ensure(n));
    SALTY_TRY_CUDA(E, cen4.ensure(n));
    for (int i = 0; i < 2; ++i) {
        SALTY_TRY_CUDA(E, prim[i].ensure(n));
        SALTY_TRY_CUDA(E, pos_task[i].ensure(n));
        SALTY_TRY_CUDA(E, tasks[i].ensure((size_t)n + 1));
        SALTY_TRY_CUDA(E, work[i].ensure((size_t)n + 1));
    }
    SALTY_TRY_CUDA(E, bnodes.ensure((size_t)2 * n + 1));
    size_t max_large = (size_t)n / kSmall + 2;
    SALTY_TRY_CUDA(E, bins.ensure(max_large * kBinWords));
    SALTY_TRY_CUDA(E, ctr.ensure(1));
    Counters* hc = (Counters*)ctx->pinned;

    cudaEvent_t e0 = ctx->ev[0], e1 = ctx->ev[1];
    cudaEventRecord(e0, st);
    k_init_counters<<<1, 1, 0, st>>>(ctr.p);
    k_prim_setup<<<grid_for(n, 256), 256, 0, st>>>(d_pos, n, lo4.p, hi4.p, cen4.p, prim[0].p,
                                                   pos_task[0].p, ctr.p);
    k_root_init<<<1, 1, 0, st>>>(ctr.p, tasks[0].p, bnodes.p, n, 0);
    int cur = 0;
    int ntasks = 1, nlarge = (n > kSmall) ? 1 : 0;
    // binary node index ranges per level: level l holds nodes [lvl[l], lvl[l + 1])
    std::vector<int> lvl{0, 1};
    for (int level = 0; ntasks > 0; ++level) {
        if (level > 4096) return E.fail(SALTY_ERR_CAPACITY, "binary build did not terminate");
        if (nlarge > 0) {
            k_clear_bins<<<grid_for((long long)nlarge * kBinWords, 256), 256, 0, st>>>(bins.p, nlarge);
            k_bin<<<grid_for(n, 256), 256, 0, st>>>(n, pos_task[cur].p, prim[cur].p, cen4.p, lo4.p, hi4.p,
                                                    tasks[cur].p, bins.p, prm.B);
        }
        cudaMemsetAsync(&ctr.p->next_tasks, 0, sizeof(int), st);
        cudaMemsetAsync(&ctr.p->next_large, 0, sizeof(int), st);
        k_split<<<grid_for(ntasks, kSplitWarps), kSplitWarps * 32, 0, st>>>(
            tasks[cur].p, ntasks, bins.p, bnodes.p, prim[cur].p, cen4.p, lo4.p, hi4.p, prm, ctr.p,
            tasks[cur ^ 1].p, level);
        k_partition<<<grid_for(n, 256), 256, 0, st>>>(n, pos_task[cur].p, prim[cur].p, cen4.p, tasks[cur].p,
                                                      tasks[cur ^ 1].p, prim[cur ^ 1].p, pos_task[cur ^ 1].p,
                                                      prm.B, ctr.p);
        SALTY_TRY_CUDA(E, cudaMemcpyAsync(hc, ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, st));
        SALTY_TRY_CUDA(E, cudaStreamSynchronize(st));
        if (hc->error) return E.fail(SALTY_ERR_CUDA, "BVH partition disagreed with its bins at level %d", level);
        ntasks = hc->next_tasks;
        nlarge = hc->next_large;
        if (hc->nodes > lvl.back()) lvl.push_back(hc->nodes);
        cur ^= 1;
    }
    SALTY_TRY_CUDA(E, cudaGetLastError());
    const int n_binary = hc->nodes;
    const int bdepth = hc->depth;

    // collapse: costs of every binary subtree, deepest level first, then the 8-wide nodes
    // top down
    DevBuf<CollapseDP> dp;
    SALTY_TRY_CUDA(E, dp.ensure((size_t)n_binary));
    for (int l = (int)lvl.size() - 2; l >= 0; --l) {
        const int b0 = lvl[l], b1 = lvl[l + 1];
        k_collapse_dp<<<grid_for(b1 - b0, 128), 128, 0, st>>>(bnodes.p, dp.p, b0, b1, kCollapseNodeCost,
                                                               kCollapseTriCost);
    }
    SALTY_TRY_CUDA(E, out.nodes.ensure((size_t)n + 1));
    SALTY_TRY_CUDA(E, out.tris.ensure((size_t)n * kTriFloat4));
    BNode root;
    SALTY_TRY_CUDA(E, cudaMemcpyAsync(&root, bnodes.p, sizeof(BNode), cudaMemcpyDeviceToHost, st));
    SALTY_TRY_CUDA(E, cudaStreamSynchronize(st));
    for (int a = 0; a < 3; ++a) { root_box[a] = root.lo[a]; root_box[3 + a] = root.hi[a]; }
    float rdx = root.hi[0] - root.lo[0], rdy = root.hi[1] - root.lo[1], rdz = root.hi[2] - root.lo[2];
    float root_sa = 2.0f * (rdx * rdy + rdx * rdz + rdy * rdz);
    if (!(root_sa > 0.0f)) root_sa = 1.0f;
    int2 w0 = make_int2(0, 0);
    SALTY_TRY_CUDA(E, cudaMemcpyAsync(work[0].p, &w0, sizeof(int2), cudaMemcpyHostToDevice, st));
    {
        int one = 1;
        SALTY_TRY_CUDA(E, cudaMemcpyAsync(&ctr.p->n8, &one, sizeof(int), cudaMemcpyHostToDevice, st));
    }
    int nwork = 1, wcur = 0, depth8 = 0;
    while (nwork > 0) {
        cudaMemsetAsync(&ctr.p->next_work, 0, sizeof(int), st);
        k_collapse<<<grid_for(nwork, 128), 128, 0, st>>>(bnodes.p, nwork, work[wcur].p, out.nodes.p,
                                                         out.tris.p, prim[cur].p, d_pos,
                                                         work[wcur ^ 1].p, ctr.p, root_sa, dp.p);
        SALTY_TRY_CUDA(E, cudaMemcpyAsync(hc, ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, st));
        SALTY_TRY_CUDA(E, cudaStreamSynchronize(st));
        nwork = hc->next_work;
        wcur ^= 1;
        ++depth8;
        if (depth8 > 4096) return E.fail(SALTY_ERR_CAPACITY, "collapse did not terminate");
    }
    cudaEventRecord(e1, st);
    SALTY_TRY_CUDA(E, cudaEventSynchronize(e1));
    SALTY_TRY_CUDA(E, cudaGetLastError());
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (hc->ntris != n) return E.fail(SALTY_ERR_CUDA, "collapse wrote %d of %d triangles", hc->ntris, n);
    out.n_nodes = hc->n8;
    out.n_tris = n;
    out.depth = depth8;
    out.built = true;
    static std::atomic<uint64_t> builds{0};
    out.generation = ++builds;  // unique in the process
    out.info.n_nodes = hc->n8;
    out.info.n_binary = n_binary;
    out.info.depth = depth8;
    out.info.binary_depth = bdepth;
    out.info.sah_cost = hc->sah;
    out.info.build_ms = ms;
    return SALTY_OK;
}

}  // namespace salty
