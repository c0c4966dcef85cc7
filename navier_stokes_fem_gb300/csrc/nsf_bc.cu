// Time-dependent Dirichlet data evaluated on the device.
//
// The reference's boundary expressions (cpp/expression.cpp) accept the variable t (cpp/expression.cpp:167-177),
// but its imposeVelocityDirichlet (include/assembly.h:1559-1579) hands them x and y only, once per step on the
// host, in float.  Here a mesh's expressions may use t: they are compiled on the host into postfix programs
// (nsfhost::Expression::compile) and evaluated in FP64 on the device at the start of every step, at the time the
// step ends, t = t0 + k dt for step k.  One thread per distinct Dirichlet node walks that node's listed
// occurrences in order, so the imposed value is the last occurrence's and the lift weight the sum over its
// occurrences, as the constant data of nsf_sim_setup are formed (a node listed twice has its lift subtracted
// twice, include/assembly.h:505-523).  The lifts W g of both velocity channels and of the pressure are then
// recomputed by the CSR product with the Dirichlet weight matrices: three products and one small kernel per step.
#include "nsf_internal.cuh"

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <unordered_map>

namespace nsf {

namespace {

// FP64 evaluation of one program; the host has checked its length and stack depth.  The _rn intrinsics keep the
// compiler from contracting a product and a sum of different ops into one FMA, so each op rounds as on the host.
__device__ double bc_run(const BcProgram& p, double x, double y, double t) {
    double st[nsfhost::kBcMaxStack];
    int sp = 0;
    for (int i = 0; i < p.n; ++i) {
        switch (p.op[i]) {
            case nsfhost::kOpConst: st[sp++] = p.c[i]; break;
            case nsfhost::kOpX: st[sp++] = x; break;
            case nsfhost::kOpY: st[sp++] = y; break;
            case nsfhost::kOpT: st[sp++] = t; break;
            case nsfhost::kOpNeg: st[sp - 1] = -st[sp - 1]; break;
            case nsfhost::kOpAdd: --sp; st[sp - 1] = __dadd_rn(st[sp - 1], st[sp]); break;
            case nsfhost::kOpSub: --sp; st[sp - 1] = __dsub_rn(st[sp - 1], st[sp]); break;
            case nsfhost::kOpMul: --sp; st[sp - 1] = __dmul_rn(st[sp - 1], st[sp]); break;
            case nsfhost::kOpDiv: --sp; st[sp - 1] = __ddiv_rn(st[sp - 1], st[sp]); break;
            case nsfhost::kOpPow: --sp; st[sp - 1] = pow(st[sp - 1], st[sp]); break;
            case nsfhost::kOpSin: st[sp - 1] = sin(st[sp - 1]); break;
            case nsfhost::kOpCos: st[sp - 1] = cos(st[sp - 1]); break;
            default: break;
        }
    }
    return st[0];
}

// Per distinct Dirichlet node: imposed values (last occurrence) and lift weights (sum of the occurrences).
// progB == nullptr: one channel (the pressure).
__global__ void bc_update_kernel(int nNodes, const int* __restrict__ node, const int* __restrict__ occStart,
                                 const int* __restrict__ progA, const int* __restrict__ progB,
                                 const BcProgram* __restrict__ progs, const float2* __restrict__ xy, double t,
                                 double* gA, double* gB, double* sumA, double* sumB) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nNodes) return;
    const int nd = node[i];
    const float2 c = xy[nd];
    const double x = c.x, y = c.y;
    double va = 0, vb = 0, sa = 0, sb = 0;
    for (int k = occStart[i]; k < occStart[i + 1]; ++k) {
        va = bc_run(progs[progA[k]], x, y, t);
        sa += va;
        if (progB) {
            vb = bc_run(progs[progB[k]], x, y, t);
            sb += vb;
        }
    }
    gA[nd] = va;
    sumA[nd] = sa;
    if (progB) {
        gB[nd] = vb;
        sumB[nd] = sb;
    }
}

// Velocity Dirichlet values on the resident field's Dirichlet rows (imposeVelocityDirichlet).
__global__ void bc_impose_kernel(int n, const unsigned char* __restrict__ mask, const double* __restrict__ g,
                                 double* __restrict__ w) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && mask[i]) w[i] = g[i];
}

// The distinct nodes of an occurrence list in order of first appearance, each with its occurrences in listed
// order: node[], occStart[] (CSR) and the occurrence indices in that grouping.
void group_occurrences(const std::vector<int>& occ, std::vector<int>& node, std::vector<int>& start,
                       std::vector<int>& order) {
    std::unordered_map<int, int> slot;
    std::vector<std::vector<int>> lists;
    for (int k = 0; k < (int)occ.size(); ++k) {
        auto it = slot.find(occ[k]);
        if (it == slot.end()) {
            it = slot.emplace(occ[k], (int)node.size()).first;
            node.push_back(occ[k]);
            lists.emplace_back();
        }
        lists[it->second].push_back(k);
    }
    start.assign(1, 0);
    for (const auto& l : lists) {
        order.insert(order.end(), l.begin(), l.end());
        start.push_back((int)order.size());
    }
}

}  // namespace

void bc_update_launch(SimState& S, const MeshDev& m, Csr* mats, double t, cudaStream_t s) {
    if (S.nBcNodeV > 0) {
        bc_update_kernel<<<(S.nBcNodeV + 127) / 128, 128, 0, s>>>(
            S.nBcNodeV, S.bcNodeV.get(), S.bcOccStartV.get(), S.bcProgU.get(), S.bcProgV.get(), S.bcProg.get(),
            m.xy.get(), t, S.gV[0].get(), S.gV[1].get(), S.gSumV[0].get(), S.gSumV[1].get());
        NSF_CUDA(cudaGetLastError());
        count_launch();
    }
    if (S.nBcNodeP > 0) {
        bc_update_kernel<<<(S.nBcNodeP + 127) / 128, 128, 0, s>>>(
            S.nBcNodeP, S.bcNodeP.get(), S.bcOccStartP.get(), S.bcProgP.get(), nullptr, S.bcProg.get(), m.xy.get(), t,
            S.gP.get(), nullptr, S.gSumP.get(), nullptr);
        NSF_CUDA(cudaGetLastError());
        count_launch();
    }
    for (int ch = 0; ch < 2; ++ch) spmv_launch(mats[NSF_VELOCITY_LIFT], S.gSumV[ch].get(), S.liftV[ch].get(), s);
    spmv_launch(mats[NSF_PRESSURE_LIFT], S.gSumP.get(), S.liftP.get(), s);
}

void bc_set_programs(SimState& S, const MeshDev& m, Csr* mats, int nExpressions, const char* const* expressions,
                     const int* velocityU, const int* velocityV, const int* pressure, double t0, cudaStream_t s) {
    const int nU = (int)S.hOccV.size(), nP = (int)S.hOccP.size();
    if (nExpressions <= 0 || !expressions) throw bad_arg("no expressions given");
    if ((nU > 0 && (!velocityU || !velocityV)) || (nP > 0 && !pressure)) throw bad_arg("null expression index array");
    if (!std::isfinite(t0)) throw bad_arg("t0 must be finite");
    std::vector<BcProgram> progs(nExpressions);
    for (int e = 0; e < nExpressions; ++e) {
        if (!expressions[e]) throw bad_arg("null expression " + std::to_string(e));
        std::vector<int> ops;
        std::vector<double> consts;
        int depth = 0;
        try {
            depth = nsfhost::Expression(expressions[e]).compile(ops, consts);
        } catch (const std::exception& err) {
            throw bad_arg("expression " + std::to_string(e) + " (\"" + expressions[e] + "\"): " + err.what());
        }
        if ((int)ops.size() > nsfhost::kBcMaxOps || depth > nsfhost::kBcMaxStack)
            throw bad_arg("expression " + std::to_string(e) + " is longer than the device evaluator holds (" +
                          std::to_string(nsfhost::kBcMaxOps) + " operations, stack depth " +
                          std::to_string(nsfhost::kBcMaxStack) + ")");
        BcProgram& p = progs[e];
        p = BcProgram{};
        p.n = (int)ops.size();
        for (int i = 0; i < p.n; ++i) {
            p.op[i] = ops[i];
            p.c[i] = consts[i];
        }
    }
    auto check = [&](const int* idx, int n, const char* what) {
        for (int k = 0; k < n; ++k)
            if (idx[k] < 0 || idx[k] >= nExpressions)
                throw bad_arg(std::string(what) + " expression index out of range at occurrence " + std::to_string(k));
    };
    check(velocityU, nU, "velocity u");
    check(velocityV, nU, "velocity v");
    check(pressure, nP, "pressure");

    std::vector<int> node, start, order;
    group_occurrences(S.hOccV, node, start, order);
    std::vector<int> pu(order.size()), pv(order.size());
    for (size_t k = 0; k < order.size(); ++k) {
        pu[k] = velocityU[order[k]];
        pv[k] = velocityV[order[k]];
    }
    S.nBcNodeV = (int)node.size();
    S.bcNodeV.upload(node.data(), node.size(), s);
    S.bcOccStartV.upload(start.data(), start.size(), s);
    S.bcProgU.upload(pu.data(), pu.size(), s);
    S.bcProgV.upload(pv.data(), pv.size(), s);
    node.clear();
    start.clear();
    order.clear();
    group_occurrences(S.hOccP, node, start, order);
    std::vector<int> pp(order.size());
    for (size_t k = 0; k < order.size(); ++k) pp[k] = pressure[order[k]];
    S.nBcNodeP = (int)node.size();
    S.bcNodeP.upload(node.data(), node.size(), s);
    S.bcOccStartP.upload(start.data(), start.size(), s);
    S.bcProgP.upload(pp.data(), pp.size(), s);
    S.bcProg.upload(progs.data(), progs.size(), s);
    for (int ch = 0; ch < 2; ++ch) {
        S.gSumV[ch].alloc(m.nNodes);
        S.gSumV[ch].zero(s);
    }
    S.gSumP.alloc(m.nP);
    S.gSumP.zero(s);
    // the data at t0, imposed on the resident velocity field as the set-up imposes the constant data
    bc_update_launch(S, m, mats, t0, s);
    for (int ch = 0; ch < 2; ++ch) {
        bc_impose_kernel<<<(m.nNodes + 255) / 256, 256, 0, s>>>(m.nNodes, S.bcV.get(), S.gV[ch].get(),
                                                               S.uv.get() + (size_t)ch * m.nNodes);
        NSF_CUDA(cudaGetLastError());
        count_launch();
    }
    NSF_CUDA(cudaStreamSynchronize(s));
    S.bcTimeDependent = true;
    S.t0 = t0;
    S.steps = 0;
}

}  // namespace nsf
