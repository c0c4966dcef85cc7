#include "expression.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <vector>

namespace nsfhost {

struct Expression::Node {
    enum Kind { Num, Var, Neg, Add, Sub, Mul, Div, Pow, Sin, Cos } kind;
    double value = 0;
    char var = 0;
    std::shared_ptr<Node> a, b;
};

namespace {

using NodeP = std::shared_ptr<Expression::Node>;

struct Tok {
    enum Kind { Num, Var, Op, Fn, End } kind;
    double value = 0;
    char c = 0;          // operator char, variable name, or 's'/'c' for sin/cos
};

std::vector<Tok> tokenize(const std::string& s) {
    std::vector<Tok> out;
    size_t i = 0;
    while (i < s.size()) {
        const char c = s[i];
        if (std::isspace((unsigned char)c)) { ++i; continue; }
        if (strchr("+-*/^()", c)) { out.push_back({Tok::Op, 0, c}); ++i; continue; }
        if (s.compare(i, 3, "sin") == 0) { out.push_back({Tok::Fn, 0, 's'}); i += 3; continue; }
        if (s.compare(i, 3, "cos") == 0) { out.push_back({Tok::Fn, 0, 'c'}); i += 3; continue; }
        if (c == 'E') { out.push_back({Tok::Num, M_E, 0}); ++i; continue; }
        if (s.compare(i, 2, "Pi") == 0) { out.push_back({Tok::Num, M_PI, 0}); i += 2; continue; }
        if (std::isdigit((unsigned char)c) || c == '.') {
            char* e = nullptr;
            const double v = strtod(s.c_str() + i, &e);
            if (e == s.c_str() + i) break;
            out.push_back({Tok::Num, v, 0});
            i = (size_t)(e - s.c_str());
            continue;
        }
        if (c == 'x' || c == 'y' || c == 'z' || c == 't') { out.push_back({Tok::Var, 0, c}); ++i; continue; }
        throw std::runtime_error("Error while parsing expression: " + s + ". Unexpected symbol: " + std::string(1, c) +
                                 " at " + std::to_string(i));
    }
    out.push_back({Tok::End, 0, 0});
    return out;
}

struct Parser {
    const std::vector<Tok>& t;
    const std::string& text;
    size_t i = 0;

    bool isOp(char c) const { return t[i].kind == Tok::Op && t[i].c == c; }
    NodeP make(Expression::Node::Kind k, NodeP a = nullptr, NodeP b = nullptr) {
        auto n = std::make_shared<Expression::Node>();
        n->kind = k;
        n->a = std::move(a);
        n->b = std::move(b);
        return n;
    }
    [[noreturn]] void fail(const char* why) { throw std::runtime_error(std::string(why) + ": " + text); }

    NodeP atom() {
        const Tok& k = t[i];
        if (k.kind == Tok::Num) { ++i; auto n = make(Expression::Node::Num); n->value = k.value; return n; }
        if (k.kind == Tok::Var) { ++i; auto n = make(Expression::Node::Var); n->var = k.c; return n; }
        if (k.kind == Tok::Fn) {
            ++i;
            if (!isOp('(')) fail("Error parsing expression. Functions must be surrounded by ()");
            NodeP arg = atom();
            return make(k.c == 's' ? Expression::Node::Sin : Expression::Node::Cos, arg);
        }
        if (isOp('(')) {
            ++i;
            NodeP v = sum();
            if (!isOp(')')) fail("Error parsing expression. Mismatched brackets.");
            ++i;
            return v;
        }
        fail("Wrong expression");
    }
    NodeP power() {
        NodeP v = atom();
        while (isOp('^')) {
            ++i;
            NodeP e;
            if (isOp('-')) { ++i; e = make(Expression::Node::Neg, power()); }
            else e = atom();
            v = make(Expression::Node::Pow, v, e);
        }
        return v;
    }
    NodeP unary() {
        if (isOp('-')) { ++i; return make(Expression::Node::Neg, unary()); }
        return power();
    }
    NodeP product() {
        NodeP v = unary();
        while (isOp('*') || isOp('/')) {
            const char c = t[i++].c;
            v = make(c == '*' ? Expression::Node::Mul : Expression::Node::Div, v, unary());
        }
        return v;
    }
    NodeP sum() {
        NodeP v = product();
        while (isOp('+') || isOp('-')) {
            const char c = t[i++].c;
            v = make(c == '+' ? Expression::Node::Add : Expression::Node::Sub, v, product());
        }
        return v;
    }
};

double eval(const Expression::Node& n, const std::map<char, double>& vars) {
    using K = Expression::Node;
    switch (n.kind) {
        case K::Num: return n.value;
        case K::Var: {
            auto it = vars.find(n.var);
            if (it == vars.end()) throw std::runtime_error(std::string("Missing variable: ") + n.var);
            return it->second;
        }
        case K::Neg: return -eval(*n.a, vars);
        case K::Add: return eval(*n.a, vars) + eval(*n.b, vars);
        case K::Sub: return eval(*n.a, vars) - eval(*n.b, vars);
        case K::Mul: return eval(*n.a, vars) * eval(*n.b, vars);
        case K::Div: return eval(*n.a, vars) / eval(*n.b, vars);
        case K::Pow: return std::pow(eval(*n.a, vars), eval(*n.b, vars));
        case K::Sin: return std::sin(eval(*n.a, vars));
        case K::Cos: return std::cos(eval(*n.a, vars));
    }
    return 0;
}

// Post-order walk: operands before their operator.  Returns the stack depth the subtree needs.
int emit(const Expression::Node& n, std::vector<int>& ops, std::vector<double>& consts) {
    using K = Expression::Node;
    auto push = [&](int op, double c = 0.0) { ops.push_back(op); consts.push_back(c); };
    switch (n.kind) {
        case K::Num: push(kOpConst, n.value); return 1;
        case K::Var:
            if (n.var == 'x') push(kOpX);
            else if (n.var == 'y') push(kOpY);
            else if (n.var == 't') push(kOpT);
            else throw std::runtime_error(std::string("Missing variable: ") + n.var);
            return 1;
        case K::Neg: case K::Sin: case K::Cos: {
            const int d = emit(*n.a, ops, consts);
            push(n.kind == K::Neg ? kOpNeg : n.kind == K::Sin ? kOpSin : kOpCos);
            return d;
        }
        default: {
            const int da = emit(*n.a, ops, consts);
            const int db = emit(*n.b, ops, consts);
            const int op = n.kind == K::Add ? kOpAdd : n.kind == K::Sub ? kOpSub : n.kind == K::Mul ? kOpMul
                         : n.kind == K::Div ? kOpDiv : kOpPow;
            push(op);
            return std::max(da, db + 1);
        }
    }
}

}  // namespace

double run_program(const std::vector<int>& ops, const std::vector<double>& consts, double x, double y, double t) {
    std::vector<double> st;
    st.reserve(kBcMaxStack);
    for (size_t i = 0; i < ops.size(); ++i) {
        const int op = ops[i];
        if (op <= kOpT) {
            st.push_back(op == kOpConst ? consts[i] : op == kOpX ? x : op == kOpY ? y : t);
            continue;
        }
        if (op == kOpNeg || op == kOpSin || op == kOpCos) {
            double& a = st.back();
            a = op == kOpNeg ? -a : op == kOpSin ? std::sin(a) : std::cos(a);
            continue;
        }
        const double b = st.back();
        st.pop_back();
        double& a = st.back();
        switch (op) {
            case kOpAdd: a = a + b; break;
            case kOpSub: a = a - b; break;
            case kOpMul: a = a * b; break;
            case kOpDiv: a = a / b; break;
            default: a = std::pow(a, b); break;
        }
    }
    return st.empty() ? 0.0 : st.front();
}

int Expression::compile(std::vector<int>& ops, std::vector<double>& consts) const {
    return emit(*root_, ops, consts);
}

Expression::Expression(const std::string& text) : text_(text) {
    const std::vector<Tok> toks = tokenize(text);
    Parser p{toks, text_};
    root_ = p.sum();
    if (toks[p.i].kind != Tok::End) throw std::runtime_error("Wrong expression: " + text);
}

double Expression::evaluate(const std::map<char, double>& vars) const { return eval(*root_, vars); }

}  // namespace nsfhost
