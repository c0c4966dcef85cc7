// ORACLE (reference build) — test infrastructure only.
// A thin C entry layer around the reference's OWN KD tree: cpp/kd_tree_builder.cpp (KDTreeBuilder::build)
// and gpu_cpu_shared/kd_tree.cuh (KDTree<FemGrid2D>::findElement), compiled unchanged from the reference
// sources by oracle/Makefile into oracle/_ref/.  It exists to pin the element-lookup oracle and to write
// golden element-ID fixtures; no product code links it.  It also exposes the reference's expression evaluator
// (cpp/expression.cpp) to pin the restated boundary-condition expression language.
//
// FemGrid2D is filled through a derived class (its members are protected, include/grid.h:110-128) in
// the same order FemGrid2D::loadJSON uses (cpp/grid.cpp:25-36), so BBox2D::expand reproduces the
// reference's grid bounding box, including its max = last node behaviour.
#include "grid.h"
#include "kd_tree.cuh"
#include "kd_tree_builder.h"
#include "expression.h"
#include "error_code.h"

namespace {

struct FilledGrid : public NSFem::FemGrid2D {
    void fill(int nNodes, const float* xy, int nEl, const int* el, int nP) {
        bbox.reset();
        nodes.clear();
        elements.clear();
        elementsCount = nEl;
        velocityNodesCount = nNodes;
        pressureNodesCount = nP;
        elementSize = 6;
        nodes.reserve(2 * (size_t)nNodes);
        for (int i = 0; i < nNodes; ++i) {
            NSFem::Point2D node(xy[2 * i], xy[2 * i + 1]);
            bbox.expand(node);
            nodes.push_back(node.x);
            nodes.push_back(node.y);
        }
        elements.assign(el, el + 6 * (size_t)nEl);
    }
};

struct State {
    FilledGrid grid;
    NSFem::KDTreeCPUOwner owner;
};

}  // namespace

extern "C" {

void* ref_tree_create(int nNodes, const float* xy, int nEl, const int* el, int nP) {
    State* s = new State;
    s->grid.fill(nNodes, xy, nEl, el, nP);
    NSFem::KDTreeBuilder builder;
    s->owner = builder.buildCPUOwner(&s->grid);
    return s;
}

void ref_tree_destroy(void* h) { delete (State*)h; }

void ref_tree_locate(void* h, int n, const float* pts, int* elem, float* xi, float* eta, int* nearest) {
    State* s = (State*)h;
    const NSFem::KDTree<NSFem::FemGrid2D> tree = s->owner.getTree();
    // findElement is const and keeps its traversal stack on the stack: queries are independent
#pragma omp parallel for schedule(dynamic, 4096)
    for (int i = 0; i < n; ++i) {
        float a = 0, b = 0;
        int nn = -1;
        const int e = tree.findElement(NSFem::Point2D(pts[2 * i], pts[2 * i + 1]), a, b, nn);
        elem[i] = e;
        xi[i] = a;
        eta[i] = b;
        nearest[i] = e >= 0 ? -1 : nn;
    }
}

// The reference's boundary-condition expression (cpp/expression.cpp, Expression::init and ::evaluate), evaluated
// the way VelocityDirichlet::eval / PressureDirichlet::eval do (cpp/grid.cpp:80-94): float variables in an
// unordered_map keyed by name.  Returns 0 and the float result, 1 when init rejects the text, 2 when evaluate
// fails (an unknown variable).
int ref_expression_eval(const char* text, float x, float y, float t, float* out) {
    NSFem::Expression e;
    if (e.init(text).hasError()) return 1;
    const std::unordered_map<char, float> vars = {{'x', x}, {'y', y}, {'t', t}};
    float r = 0;
    if (e.evaluate(&vars, r).hasError()) return 2;
    *out = r;
    return 0;
}

void ref_grid_bbox(void* h, float* out4) {
    const NSFem::BBox2D& bb = ((State*)h)->grid.getBBox();
    out4[0] = bb.getMin().x;
    out4[1] = bb.getMin().y;
    out4[2] = bb.getMax().x;
    out4[3] = bb.getMax().y;
}

}  // extern "C"
