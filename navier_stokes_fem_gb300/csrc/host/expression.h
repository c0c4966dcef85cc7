// Boundary-condition expressions of the reference's mesh files (include/expression.h, cpp/expression.cpp):
// numbers, variables x y z t, constants E and Pi, binary + - * / ^, unary minus, sin(...) and cos(...).
// Precedence from low to high: + -, * /, unary minus, ^ (left associative), function call.
#pragma once
#include <map>
#include <memory>
#include <string>

namespace nsfhost {

class Expression {
public:
    // Throws std::runtime_error with the reference's messages on malformed input.
    explicit Expression(const std::string& text);
    // Evaluates in double; throws on a variable missing from `vars`.
    double evaluate(const std::map<char, double>& vars) const;
    const std::string& text() const { return text_; }

    struct Node;

private:
    std::string text_;
    std::shared_ptr<Node> root_;
};

}  // namespace nsfhost
