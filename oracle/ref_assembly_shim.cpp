// ORACLE (reference build) — test infrastructure only.
// The reference's OWN element arithmetic, compiled from its lines: the P1/P2 shape functions, the Jacobian and
// differential operator and the 7-point TriangleIntegrator (include/assembly.h:98-304), and the local mass,
// stiffness and divergence functors (include/assembly.h:725-882), and the convection functor of
// assembleConvectionMatrix (include/assembly.h:1584-1622).  oracle/Makefile (`make ref-assembly`) copies
// those line ranges verbatim into the git-ignored build folder _ref/ (checking the first and last line of
// each range) and this file includes them.  The functors are member templates of NavierStokesAssembly<P2, P1>,
// whose other members need the absent sparse_matrix_math submodule, TBB, OpenCV and nlohmann_json; here they sit
// inside ElementFunctors<VelocityShape, PressureShape>, a class template of this file that provides only the two
// template parameters their bodies name.  No product code links this: it pins the oracle's restated local matrices.
#include <algorithm>
#include <cassert>
#include <cmath>

#include "misc_common.cuh"
#include "static_matrix.h"

namespace NSFem {

#include "assembly_shapes.inc"

template <typename VelocityShape, typename PressureShape>
struct ElementFunctors {
#include "assembly_functors.inc"
};

using Functors = ElementFunctors<P2, P1>;

// The convection functor of NavierStokesAssembly::assembleConvectionMatrix (include/assembly.h:1584-1622, copied by
// `make ref-assembly` into _ref/assembly_convection.inc): a lambda over the member `currentVelocitySolution` and
// `grid.getNodesCount()`, which this class provides for one element whose six velocities sit at indexes 0..5 (u)
// and 6..11 (v).
template <typename VelocityShape>
struct ConvectionHost {
    struct Grid {
        int getNodesCount() const { return 6; }
    } grid;
    real currentVelocitySolution[12];
    void local(const real* elementNodes, StaticMatrix<real, VelocityShape::size, VelocityShape::size>& out) {
#include "assembly_convection.inc"
        const int indexes[6] = {0, 1, 2, 3, 4, 5};
        localConvection(indexes, elementNodes, out);
    }
};

}  // namespace NSFem

namespace {

template <typename M>
void store(const M& m, int rows, int cols, float* out) {
    for (int i = 0; i < rows; ++i)
        for (int j = 0; j < cols; ++j) out[i * cols + j] = m[i][j];
}

}  // namespace

extern "C" {

// Local matrices of `n` triangles, as the reference's assembly computes them in float.  vertices: per triangle
// x0 y0 x1 y1 x2 y2 (the first three element nodes, counter-clockwise).  Per triangle, row-major:
//   mass     6x6  LocalMassFunctor<P2>                  (velocity mass)
//   stiffV   6x6  LocalStiffnessFunctor<P2>             (velocity stiffness, before the dt * nu scaling)
//   stiffP   3x3  LocalStiffnessFunctor<P1>             (pressure stiffness)
//   divVx/y  3x6  LocalDivergenceFunctor<P1, P2>        (velocity divergence blocks, before the -1/dt scaling)
//   divPx/y  6x3  LocalDivergenceFunctor<P2, P1>        (pressure gradient blocks, before the -dt scaling)
void ref_local_matrices(int n, const float* vertices, float* mass, float* stiffV, float* stiffP, float* divVx,
                        float* divVy, float* divPx, float* divPy) {
    using namespace NSFem;
    const Functors::LocalMassFunctor<P2> fm;
    const Functors::LocalStiffnessFunctor<P2> fkv;
    const Functors::LocalStiffnessFunctor<P1> fkp;
    const Functors::LocalDivergenceFunctor<P1, P2> fdv;
    const Functors::LocalDivergenceFunctor<P2, P1> fdp;
    const int unusedIndexes[6] = {0, 1, 2, 3, 4, 5};
    for (int e = 0; e < n; ++e) {
        real nodes[12] = {};
        for (int k = 0; k < 6; ++k) nodes[k] = vertices[6 * e + k];
        StaticMatrix<real, 6, 6> m66;
        fm(unusedIndexes, nodes, m66);
        store(m66, 6, 6, mass + 36 * e);
        StaticMatrix<real, 6, 6> k66;
        fkv(unusedIndexes, nodes, k66);
        store(k66, 6, 6, stiffV + 36 * e);
        StaticMatrix<real, 3, 3> k33;
        fkp(unusedIndexes, nodes, k33);
        store(k33, 3, 3, stiffP + 9 * e);
        StaticMatrix<real, 3, 6> dx, dy;
        fdv(unusedIndexes, nodes, dx, dy);
        store(dx, 3, 6, divVx + 18 * e);
        store(dy, 3, 6, divVy + 18 * e);
        StaticMatrix<real, 6, 3> gx, gy;
        fdp(unusedIndexes, nodes, gx, gy);
        store(gx, 6, 3, divPx + 18 * e);
        store(gy, 6, 3, divPy + 18 * e);
    }
}

// The local convection matrix (6x6, row-major) of `n` triangles with the nodal velocities vel (per triangle u0..u5,
// v0..v5), as the reference's assembleConvectionMatrix computes it in float.
void ref_local_convection(int n, const float* vertices, const float* vel, float* conv) {
    using namespace NSFem;
    ConvectionHost<P2> host;
    for (int e = 0; e < n; ++e) {
        real nodes[12] = {};
        for (int k = 0; k < 6; ++k) nodes[k] = vertices[6 * e + k];
        for (int k = 0; k < 12; ++k) host.currentVelocitySolution[k] = vel[12 * e + k];
        StaticMatrix<real, 6, 6> c;
        host.local(nodes, c);
        store(c, 6, 6, conv + 36 * e);
    }
}

}  // extern "C"
