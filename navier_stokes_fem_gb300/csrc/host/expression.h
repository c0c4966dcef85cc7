// Boundary-condition expressions of the reference's mesh files (include/expression.h, cpp/expression.cpp):
// numbers, variables x y z t, constants E and Pi, binary + - * / ^, unary minus, sin(...) and cos(...).
// Precedence from low to high: + -, * /, unary minus, ^ (left associative), function call.
#pragma once
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace nsfhost {

// Postfix program of an expression for the device-side evaluator of time-dependent Dirichlet data: kOpConst
// pushes its constant, kOpX/kOpY/kOpT push a variable, the unary ops replace the top of the stack, the binary ops
// pop the right operand and replace the left one.
enum BcOp : int { kOpConst = 0, kOpX, kOpY, kOpT, kOpNeg, kOpAdd, kOpSub, kOpMul, kOpDiv, kOpPow, kOpSin, kOpCos };
constexpr int kBcMaxOps = 64;     // program length the device evaluator holds
constexpr int kBcMaxStack = 16;   // stack depth it holds

// Host evaluation of a compiled program, op for op as the device evaluator runs it (the programs' own check).
double run_program(const std::vector<int>& ops, const std::vector<double>& consts, double x, double y, double t);

class Expression {
public:
    // Throws std::runtime_error with the reference's messages on malformed input.
    explicit Expression(const std::string& text);
    // Evaluates in double; throws on a variable missing from `vars`.
    double evaluate(const std::map<char, double>& vars) const;
    const std::string& text() const { return text_; }
    // Appends the postfix program (op codes and, per op, the constant of a kOpConst) and returns the stack depth
    // it needs.  Throws std::runtime_error on a variable other than x, y and t.
    int compile(std::vector<int>& ops, std::vector<double>& consts) const;

    struct Node;

private:
    std::string text_;
    std::shared_ptr<Node> root_;
};

}  // namespace nsfhost
