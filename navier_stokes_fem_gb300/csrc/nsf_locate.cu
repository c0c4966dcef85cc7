// Point location and semi-Lagrangian advection on the GPU.
//
// Replaces the reference's CPU-built KD tree (cpp/kd_tree_builder.cpp:81-149) and its advect kernel
// (gpu/advection.cu:14-57, driven by cpp/gpu_simulation_device.cpp:91-131).
//
// Tree: triangles are ordered by the Morton code of their centroid (a radix sort on the GPU), cut into
// leaves of kLeafSize consecutive triangles, and the leaves form an implicit complete binary tree whose
// nodes carry the union of their triangles' closed vertex bounding boxes.  No pointers, no recursion, and
// the build is three data-parallel passes.
//
// Query semantics match the reference exactly: its tree sends every triangle whose closed vertex box holds
// the point into the point's leaf (straddlers go to both sides, kd_tree_builder.cpp:134-141), and each leaf
// lists triangles in ascending index, so its "first triangle in the leaf passing isPointInTriagle" is the
// LOWEST-index triangle whose box holds the point and whose predicate passes.  This kernel visits every
// node whose box holds the point and keeps that minimum.  The predicate is evaluated with IEEE
// round-to-nearest float intrinsics in the reference's operation order (kd_tree_common.cuh:38-60), so
// element ids and (xi, eta) are bit-identical.  When no triangle contains the point, the nearest mesh node
// (all six nodes of each triangle, as nearestNeghbourProcessLeaf does, kd_tree.cuh:149-169) is found by a
// box-distance branch and bound; equal distances resolve to the lowest node index.
#include "nsf_internal.cuh"

#include <cub/device/device_radix_sort.cuh>

#include "nsf_locate_device.cuh"

#include <cfloat>
#include <climits>

namespace nsf {

__global__ void locate_kernel(TreeView t, int n, const float2* __restrict__ pts, int* elem, float* xiOut,
                              float* etaOut, int* nearestOut) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float2 p = pts[i];
        float xi = 0.f, eta = 0.f;
        int nn = -1;
        const int e = locate_point(t, p.x, p.y, xi, eta, nn);
        elem[i] = e;
        xiOut[i] = xi;
        etaOut[i] = eta;
        nearestOut[i] = e >= 0 ? -1 : nn;
    }
}

// Back-trace x - dt*u in float (the reference's Point2D arithmetic, include/assembly.h:1690-1692), locate,
// interpolate in double.
__global__ void advect_kernel(TreeView t, int nNodes, float fdt, const double* __restrict__ u,
                              const double* __restrict__ v, double* __restrict__ uo, double* __restrict__ vo) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nNodes; i += gridDim.x * blockDim.x) {
        const float2 pos = t.xy[i];
        const double ui = u[i], vi = v[i];
        const float px = __fsub_rn(pos.x, __fmul_rn((float)ui, fdt));
        const float py = __fsub_rn(pos.y, __fmul_rn((float)vi, fdt));
        float xi = 0.f, eta = 0.f;
        int nn = -1;
        const int e = locate_point(t, px, py, xi, eta, nn);
        if (e >= 0) {
            double N[6];
            p2_eval_d((double)xi, (double)eta, N);
            const int* en = t.el + 6 * (size_t)e;
            double su = 0.0, sv = 0.0;
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                const int nd = en[k];
                su = __dadd_rn(su, __dmul_rn(N[k], u[nd]));
                sv = __dadd_rn(sv, __dmul_rn(N[k], v[nd]));
            }
            uo[i] = su;
            vo[i] = sv;
        } else {
            // nn stays -1 only for a non-finite departure point (a non-finite velocity): keep the node's value
            const int src = nn >= 0 ? nn : i;
            uo[i] = u[src];
            vo[i] = v[src];
        }
    }
}

__global__ void advect_f32_kernel(TreeView t, int nNodes, float fdt, const float* __restrict__ u,
                                  const float* __restrict__ v, float* __restrict__ uo, float* __restrict__ vo) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nNodes; i += gridDim.x * blockDim.x) {
        const float2 pos = t.xy[i];
        const float px = __fsub_rn(pos.x, __fmul_rn(u[i], fdt));
        const float py = __fsub_rn(pos.y, __fmul_rn(v[i], fdt));
        float xi = 0.f, eta = 0.f;
        int nn = -1;
        const int e = locate_point(t, px, py, xi, eta, nn);
        if (e >= 0) {
            float N[6];
            p2_eval_f(xi, eta, N);
            const int* en = t.el + 6 * (size_t)e;
            float su = 0.f, sv = 0.f;
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                su = __fadd_rn(su, __fmul_rn(N[k], u[en[k]]));
                sv = __fadd_rn(sv, __fmul_rn(N[k], v[en[k]]));
            }
            uo[i] = su;
            vo[i] = sv;
        } else {
            const int src = nn >= 0 ? nn : i;
            uo[i] = u[src];
            vo[i] = v[src];
        }
    }
}

// ---------------------------------------------------------------------------------------------------
// build
// ---------------------------------------------------------------------------------------------------
__device__ __forceinline__ unsigned spread_bits(unsigned v) {   // 16 -> 32 bits, interleaving zeros
    v &= 0xFFFFu;
    v = (v | (v << 8)) & 0x00FF00FFu;
    v = (v | (v << 4)) & 0x0F0F0F0Fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

__global__ void morton_kernel(int nEl, const float2* __restrict__ xy, const int* __restrict__ el, float4 bb,
                              unsigned long long* keys) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nEl; e += gridDim.x * blockDim.x) {
        const int* en = el + 6 * (size_t)e;
        const float2 A = xy[en[0]], B = xy[en[1]], C = xy[en[2]];
        const float cx = (A.x + B.x + C.x) * (1.0f / 3.0f), cy = (A.y + B.y + C.y) * (1.0f / 3.0f);
        const float sx = bb.z > bb.x ? (cx - bb.x) / (bb.z - bb.x) : 0.f;
        const float sy = bb.w > bb.y ? (cy - bb.y) / (bb.w - bb.y) : 0.f;
        const unsigned qx = (unsigned)fminf(fmaxf(sx * 65535.f, 0.f), 65535.f);
        const unsigned qy = (unsigned)fminf(fmaxf(sy * 65535.f, 0.f), 65535.f);
        const unsigned code = spread_bits(qx) | (spread_bits(qy) << 1);
        keys[e] = ((unsigned long long)code << 32) | (unsigned)e;
    }
}

__global__ void leaf_kernel(int nEl, int nLeaves, const unsigned long long* __restrict__ sorted,
                            const float2* __restrict__ xy, const int* __restrict__ el, int* tri, float4* box) {
    for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < nLeaves; l += gridDim.x * blockDim.x) {
        float4 b = make_float4(FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX);
        for (int s = 0; s < kLeafSize; ++s) {
            const long long k = (long long)l * kLeafSize + s;
            int e = -1;
            if (k < nEl) {
                e = (int)(sorted[k] & 0xFFFFFFFFull);
                const int* en = el + 6 * (size_t)e;
                for (int j = 0; j < 3; ++j) {
                    const float2 p = xy[en[j]];
                    b.x = fminf(b.x, p.x); b.y = fminf(b.y, p.y);
                    b.z = fmaxf(b.z, p.x); b.w = fmaxf(b.w, p.y);
                }
            }
            tri[k] = e;
        }
        box[nLeaves - 1 + l] = b;
    }
}

__global__ void level_kernel(int first, int count, float4* box) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const int nd = first + i;
        const float4 l = box[2 * nd + 1], r = box[2 * nd + 2];
        box[nd] = make_float4(fminf(l.x, r.x), fminf(l.y, r.y), fmaxf(l.z, r.z), fmaxf(l.w, r.w));
    }
}

static int blocks_for(long long n, int t) { return (int)std::max<long long>(1, std::min<long long>((n + t - 1) / t, 152LL * 64)); }

void tree_build(MeshDev& m, cudaStream_t s) {
    const int nEl = m.nEl;
    float4 bb = make_float4(FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX);
    for (int i = 0; i < m.nNodes; ++i) {
        bb.x = std::min(bb.x, m.hxy[2 * i]); bb.y = std::min(bb.y, m.hxy[2 * i + 1]);
        bb.z = std::max(bb.z, m.hxy[2 * i]); bb.w = std::max(bb.w, m.hxy[2 * i + 1]);
    }
    int leaves = 1, depth = 0;
    while ((long long)leaves * kLeafSize < nEl) { leaves <<= 1; ++depth; }
    LocateTree& t = m.tree;
    t.nLeaves = leaves;
    t.leafSize = kLeafSize;
    t.depth = depth;
    if (depth + 2 > kStack) throw Error{NSF_ERR_BAD_ARG, "mesh too large for the point-location stack"};
    DevBuf<unsigned long long> keys, sorted;
    keys.alloc(std::max(1, nEl));
    sorted.alloc(std::max(1, nEl));
    morton_kernel<<<blocks_for(nEl, 256), 256, 0, s>>>(nEl, m.xy.get(), m.el.get(), bb, keys.get());
    NSF_CUDA(cudaGetLastError());
    count_launch();
    size_t tmpBytes = 0;
    NSF_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, tmpBytes, keys.get(), sorted.get(), nEl, 0, 64, s));
    DevBuf<unsigned char> tmp;
    tmp.alloc(std::max<size_t>(tmpBytes, 1));
    NSF_CUDA(cub::DeviceRadixSort::SortKeys(tmp.get(), tmpBytes, keys.get(), sorted.get(), nEl, 0, 64, s));
    t.triSorted.alloc((size_t)leaves * kLeafSize);
    t.box.alloc((size_t)2 * leaves - 1);
    leaf_kernel<<<blocks_for(leaves, 256), 256, 0, s>>>(nEl, leaves, sorted.get(), m.xy.get(), m.el.get(),
                                                       t.triSorted.get(), t.box.get());
    NSF_CUDA(cudaGetLastError());
    count_launch();
    for (int lvl = depth - 1; lvl >= 0; --lvl) {
        const int first = (1 << lvl) - 1, count = 1 << lvl;
        level_kernel<<<blocks_for(count, 256), 256, 0, s>>>(first, count, t.box.get());
        NSF_CUDA(cudaGetLastError());
    count_launch();
    }
    NSF_CUDA(cudaStreamSynchronize(s));   // keys/sorted/tmp are released on return
}

static TreeView view(const MeshDev& m) {
    return TreeView{m.xy.get(), m.el.get(), m.tree.triSorted.get(), m.tree.box.get(), m.tree.nLeaves};
}

void locate_launch(const MeshDev& m, int n, const float2* pts, int* elem, float* xi, float* eta, int* nearest,
                   cudaStream_t s) {
    if (n <= 0) return;
    locate_kernel<<<blocks_for(n, 128), 128, 0, s>>>(view(m), n, pts, elem, xi, eta, nearest);
    NSF_CUDA(cudaGetLastError());
    count_launch();
}

void advect_launch(const MeshDev& m, double dt, const double* u, const double* v, double* uo, double* vo,
                   cudaStream_t s) {
    advect_kernel<<<blocks_for(m.nNodes, 128), 128, 0, s>>>(view(m), m.nNodes, (float)dt, u, v, uo, vo);
    NSF_CUDA(cudaGetLastError());
    count_launch();
}

void advect_f32_launch(const MeshDev& m, float dt, const float* u, const float* v, float* uo, float* vo,
                       cudaStream_t s) {
    advect_f32_kernel<<<blocks_for(m.nNodes, 128), 128, 0, s>>>(view(m), m.nNodes, dt, u, v, uo, vo);
    NSF_CUDA(cudaGetLastError());
    count_launch();
}

}  // namespace nsf
