// Device-side point location and P2 interpolation, shared by the advection kernels (nsf_locate.cu) and the
// persistent step kernel (nsf_step.cu).  See nsf_locate.cu for the tree and the query semantics.
#pragma once
#include <cfloat>
#include <climits>

namespace nsf {

constexpr int kLeafSize = 8;
constexpr int kStack = 48;

__device__ __forceinline__ float2 node_xy(const float2* xy, int i) { return xy[i]; }

// isPointInTriagle with every float operation rounded on its own (no contraction)
__device__ __forceinline__ bool point_in_triangle(float px, float py, float2 A, float2 B, float2 C, float& xi,
                                                  float& eta) {
    const float abx = __fsub_rn(B.x, A.x), aby = __fsub_rn(B.y, A.y);
    const float acx = __fsub_rn(C.x, A.x), acy = __fsub_rn(C.y, A.y);
    const float apx = __fsub_rn(px, A.x), apy = __fsub_rn(py, A.y);
    const float D = __fsub_rn(__fmul_rn(abx, acy), __fmul_rn(aby, acx));
    const float sgn = D > 0.f ? 1.f : -1.f;
    const float s1 = __fmul_rn(__fsub_rn(__fmul_rn(apx, acy), __fmul_rn(apy, acx)), sgn);
    if (s1 < 0.f || s1 > D) return false;
    const float s2 = __fmul_rn(__fsub_rn(__fmul_rn(apy, abx), __fmul_rn(apx, aby)), sgn);
    if (s2 < 0.f || s1 > __fsub_rn(D, s2)) return false;
    const float inv = __frcp_rn(fabsf(D));
    xi = __fmul_rn(s1, inv);
    eta = __fmul_rn(s2, inv);
    return true;
}

__device__ __forceinline__ bool box_holds(float4 b, float px, float py) {
    return b.x <= px && px <= b.z && b.y <= py && py <= b.w;
}

__device__ __forceinline__ float box_dist2(float4 b, float px, float py) {
    const float dx = fmaxf(fmaxf(__fsub_rn(b.x, px), __fsub_rn(px, b.z)), 0.f);
    const float dy = fmaxf(fmaxf(__fsub_rn(b.y, py), __fsub_rn(py, b.w)), 0.f);
    return __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
}

struct TreeView {
    const float2* xy;
    const int* el;
    const int* tri;
    const float4* box;
    int nLeaves;
};

// Containing element (lowest index) or -1; on -1, `nearest` holds the closest node.
__device__ __forceinline__ int locate_point(const TreeView& t, float px, float py, float& xi, float& eta, int& nearest) {
    int stack[kStack];
    int sp = 0;
    stack[sp++] = 0;
    int best = INT_MAX;
    const int firstLeaf = t.nLeaves - 1;
    while (sp > 0) {
        const int nd = stack[--sp];
        if (!box_holds(t.box[nd], px, py)) continue;
        if (nd >= firstLeaf) {
            const int* slots = t.tri + (size_t)(nd - firstLeaf) * kLeafSize;
            for (int s = 0; s < kLeafSize; ++s) {
                const int e = slots[s];
                if (e < 0) break;
                if (e >= best) continue;
                const int* en = t.el + 6 * (size_t)e;
                const float2 A = t.xy[en[0]], B = t.xy[en[1]], C = t.xy[en[2]];
                const float4 tb = make_float4(fminf(A.x, fminf(B.x, C.x)), fminf(A.y, fminf(B.y, C.y)),
                                              fmaxf(A.x, fmaxf(B.x, C.x)), fmaxf(A.y, fmaxf(B.y, C.y)));
                if (!box_holds(tb, px, py)) continue;
                float a, b;
                if (point_in_triangle(px, py, A, B, C, a, b)) { best = e; xi = a; eta = b; }
            }
        } else if (sp + 2 <= kStack) {
            stack[sp++] = 2 * nd + 2;
            stack[sp++] = 2 * nd + 1;
        }
    }
    if (best != INT_MAX) return best;

    // nearest mesh node: branch and bound on box distance, nearer child first
    float bestD = FLT_MAX;
    int bestNode = -1;
    sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const int nd = stack[--sp];
        if (box_dist2(t.box[nd], px, py) > bestD) continue;
        if (nd >= firstLeaf) {
            const int* slots = t.tri + (size_t)(nd - firstLeaf) * kLeafSize;
            for (int s = 0; s < kLeafSize; ++s) {
                const int e = slots[s];
                if (e < 0) break;
                const int* en = t.el + 6 * (size_t)e;
                for (int j = 0; j < 6; ++j) {
                    const int v = en[j];
                    const float2 q = t.xy[v];
                    const float dx = __fsub_rn(px, q.x), dy = __fsub_rn(py, q.y);
                    const float d = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
                    if (d < bestD || (d == bestD && v < bestNode)) { bestD = d; bestNode = v; }
                }
            }
        } else if (sp + 2 <= kStack) {
            const int l = 2 * nd + 1, r = 2 * nd + 2;
            const float dl = box_dist2(t.box[l], px, py), dr = box_dist2(t.box[r], px, py);
            if (dl <= dr) { stack[sp++] = r; stack[sp++] = l; }
            else { stack[sp++] = l; stack[sp++] = r; }
        }
    }
    nearest = bestNode;
    return -1;
}

// P2 shape functions (include/assembly.h:217-224) evaluated left to right with every double operation
// rounded on its own, the same sequence the oracle compiles without contraction.
__device__ __forceinline__ void p2_eval_d(double xi, double eta, double N[6]) {
    const double x2 = __dmul_rn(__dmul_rn(2.0, xi), xi);
    const double e2 = __dmul_rn(__dmul_rn(2.0, eta), eta);
    const double xe4 = __dmul_rn(__dmul_rn(4.0, xi), eta);
    N[0] = __dadd_rn(__dadd_rn(__dadd_rn(__dsub_rn(__dsub_rn(1.0, __dmul_rn(3.0, xi)), __dmul_rn(3.0, eta)), x2), xe4), e2);
    N[1] = __dsub_rn(x2, xi);
    N[2] = __dsub_rn(e2, eta);
    N[3] = xe4;
    N[4] = __dsub_rn(__dsub_rn(__dmul_rn(4.0, eta), xe4), __dmul_rn(__dmul_rn(4.0, eta), eta));
    N[5] = __dsub_rn(__dsub_rn(__dmul_rn(4.0, xi), __dmul_rn(__dmul_rn(4.0, xi), xi)), xe4);
}
__device__ __forceinline__ void p2_eval_f(float xi, float eta, float N[6]) {
    const float x2 = __fmul_rn(__fmul_rn(2.f, xi), xi);
    const float e2 = __fmul_rn(__fmul_rn(2.f, eta), eta);
    const float xe4 = __fmul_rn(__fmul_rn(4.f, xi), eta);
    N[0] = __fadd_rn(__fadd_rn(__fadd_rn(__fsub_rn(__fsub_rn(1.f, __fmul_rn(3.f, xi)), __fmul_rn(3.f, eta)), x2), xe4), e2);
    N[1] = __fsub_rn(x2, xi);
    N[2] = __fsub_rn(e2, eta);
    N[3] = xe4;
    N[4] = __fsub_rn(__fsub_rn(__fmul_rn(4.f, eta), xe4), __fmul_rn(__fmul_rn(4.f, eta), eta));
    N[5] = __fsub_rn(__fsub_rn(__fmul_rn(4.f, xi), __fmul_rn(__fmul_rn(4.f, xi), xi)), xe4);
}

}  // namespace nsf
