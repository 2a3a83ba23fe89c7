// Algebraic rewrites applied to kernel templates.
//
// Restates reference src/Simplify.cpp: constant folding in sums and products,
// flattening of nested sums/products, merging of repeated summands and
// factors, factoring out shared factors, and the rewrite of multiplications by
// -1 into negations.  Hash-ordered maps (keyed by algebraic hash) fix operand
// order, which fixes the floating-point evaluation order of the templates.
#include <algorithm>
#include <cmath>
#include <map>
#include <set>

#include "symgb/frontend.hpp"
#include "symgb/traverse.hpp"

namespace symgb {

namespace {

bool isMul(const Symbolic& x) { return x.op() == MUL || x.op() == MULC; }

template <class F>
std::vector<Symbolic> mapChildren(const Symbolic& x, F f) {
    std::vector<Symbolic> r;
    r.reserve(x.numChilds());
    for (const Symbolic& c : x) r.push_back(f(c));
    return r;
}

}  // namespace

// Product with constants (and expressions whose hash is a small integer)
// folded into one trailing constant factor (reference Simplify.cpp:13-36).
Symbolic makeMul(const std::vector<Symbolic>& childs) {
    if (childs.empty()) return Symbolic(1.0);
    std::vector<Symbolic> rest;
    double f = 1.0;
    for (const auto& c : childs) {
        if (c.op() == CONST)
            f *= c.constant();
        else if (isSmallConstant(c.ahash()))
            f *= (double)c.ahash();
        else
            rest.push_back(c);
    }
    if (f == 0.0) return Symbolic(0.0);
    if (f != 1.0) rest.push_back(Symbolic(f));
    if (rest.empty()) return Symbolic(1.0);
    if (rest.size() == 1) return rest.front();
    return Symbolic(MUL, rest);
}

// Sum with its constant operands folded into one trailing constant
// (reference Simplify.cpp:38-57).
Symbolic makeAddition(std::vector<Symbolic> operands) {
    double constant = 0.0;
    operands.erase(std::remove_if(operands.begin(), operands.end(),
                                  [&](const Symbolic& x) {
                                      if (x.op() == CONST) {
                                          constant += x.constant();
                                          return true;
                                      }
                                      return false;
                                  }),
                   operands.end());
    if (constant != 0) operands.push_back(Symbolic(constant));
    if (operands.empty()) return Symbolic(0.0);
    if (operands.size() == 1) return operands.front();
    return Symbolic(ADD, operands);
}

Symbolic makeSymbolic(OpType op, std::vector<Symbolic> operands) {
    Symbolic ret;
    switch (op) {
        case ADD: ret = makeAddition(std::move(operands)); break;
        case MUL:
        case MULC: ret = makeMul(operands); break;
        default: ret = Symbolic(op, operands);
    }
    if (isSmallConstant(ret.ahash())) return Symbolic((double)ret.ahash());
    return ret;
}

// Operands of nested sums, in pre-order; zero-hash operands are dropped
// (reference Simplify.cpp:84-105).
Symbolic flattenAdditions(const Symbolic& expr) {
    if (expr.op() != ADD) return expr;
    std::vector<Symbolic> operands;
    preOrderTraverse(expr, [&](const Symbolic& x) {
        if (!x.ahash()) return false;
        if (x.op() != ADD) {
            operands.push_back(x);
            return false;
        }
        return true;
    });
    Symbolic ret(ADD, operands);
    if (ret.ahash() == 0)
        ret = Symbolic(0.0);
    else if (ret.numChilds() == 1)
        ret = Symbolic(ret[0]);
    return ret;
}

// Factors of nested products (reference Simplify.cpp:109-129).
Symbolic flattenMultiplications(const Symbolic& expr) {
    if (!isMul(expr)) return expr;
    std::vector<Symbolic> operands;
    preOrderTraverse(expr, [&](const Symbolic& x) {
        if (isSmallConstant(x.ahash())) {
            if (x.ahash() != 1) operands.push_back(Symbolic((double)x.ahash()));
            return false;
        }
        if (!isMul(x)) {
            operands.push_back(x);
            return false;
        }
        return true;
    });
    return makeSymbolic(MUL, operands);
}

namespace {

Symbolic makePower(const Symbolic& x, double d) {
    if (x.op() == CONST) return Symbolic(std::pow(x.constant(), d));
    if (x.op() == POW && x[1].op() == CONST) return Symbolic(POW, x[0], Symbolic(d * x[1].constant()));
    return Symbolic(POW, x, Symbolic(d));
}

// Products, quotients and square roots as one product of powers
// (reference Simplify.cpp:145-189).
Symbolic flattenDivAndMul(const Symbolic& expr) {
    std::vector<Symbolic> childs;
    switch (expr.op()) {
        case MUL:
        case MULC:
            for (auto& c : mapChildren(expr, [](const Symbolic& y) { return flattenDivAndMul(y); })) {
                if (isMul(c))
                    for (auto& cc : c) childs.push_back(cc);
                else
                    childs.push_back(c);
            }
            break;
        case SQRT: {
            Symbolic rad = flattenDivAndMul(expr[0]);
            if (isMul(rad))
                for (auto& c : rad) childs.push_back(makePower(c, 0.5));
            else
                childs.push_back(makePower(rad, 0.5));
            break;
        }
        case DIV: {
            Symbolic nom = flattenDivAndMul(expr[0]);
            Symbolic den = flattenDivAndMul(expr[1]);
            if (isMul(nom))
                for (auto& c : nom) childs.push_back(c);
            else
                childs.push_back(nom);
            if (isMul(den))
                for (auto& c : den) childs.push_back(makePower(c, -1.0));
            else
                childs.push_back(makePower(den, -1.0));
            break;
        }
        default: return expr;
    }
    return makeMul(childs);
}

}  // namespace

// Merges equal factors into powers and rebuilds numerator / denominator
// (reference Simplify.cpp:191-263).
Symbolic optimizeProducts(const Symbolic& x) {
    Symbolic xf = flattenDivAndMul(x);
    if (!isMul(xf)) return x;
    std::map<Symbolic, double, AlgebraicHashLess> factors;
    for (auto& c : xf) {
        if (c.op() == POW)
            factors[c[0]] += c[1].constant();
        else
            factors[c] += 1.0;
    }
    std::vector<Symbolic> nom, den, nomR, denR;
    double f = 1.0;
    for (auto& c : factors) {
        if (c.first.op() == CONST) {
            f *= std::pow(c.first.constant(), c.second);
        } else if (c.second < 0) {
            if (std::floor(c.second) == c.second) {
                for (int i = 0; i < std::floor(-c.second); ++i) den.push_back(c.first);
            } else if (std::floor(2 * c.second) == 2 * c.second) {
                for (int i = 0; i < std::floor(-c.second); ++i) den.push_back(c.first);
                denR.push_back(c.first);
            }
        } else if (c.second > 0) {
            if (std::floor(c.second) == c.second) {
                for (int i = 0; i < std::floor(c.second); ++i) nom.push_back(c.first);
            } else if (std::floor(2 * c.second) == 2 * c.second) {
                for (int i = 0; i < std::floor(c.second); ++i) nom.push_back(c.first);
                nomR.push_back(c.first);
            }
        }
    }
    if (!nomR.empty()) {
        if (denR.empty())
            nom.emplace_back(SQRT, makeMul(nomR));
        else
            nom.emplace_back(SQRT, makeMul(nomR) / makeMul(denR));
    } else if (!denR.empty()) {
        den.emplace_back(SQRT, makeMul(denR));
    }
    if (f != 1.0) nom.push_back(Symbolic(f));
    if (nom.empty()) nom.push_back(Symbolic(1.0));
    Symbolic ret = makeMul(nom);
    if (!ret.ahash()) return Symbolic(0.0);
    if (!den.empty()) ret = ret / makeMul(den);
    return ret;
}

namespace {

// c * (product) with all constant factors pulled into c
// (reference Simplify.cpp:265-281).
Symbolic pullConstant(const Symbolic& x0) {
    Symbolic x = flattenMultiplications(x0);
    if (x.op() == MULC) return x;
    if (x.op() != MUL) return Symbolic(MULC, Symbolic(1.0), x);
    double f = 1.0;
    std::vector<Symbolic> childs;
    for (auto& c : x) {
        if (c.op() == CONST)
            f *= c.constant();
        else
            childs.push_back(c);
    }
    return Symbolic(MULC, Symbolic(f), makeSymbolic(MUL, childs));
}

}  // namespace

// Collects equal summands with their coefficients (reference Simplify.cpp:283-307).
Symbolic optimizeSum(const Symbolic& x0) {
    Symbolic x = flattenAdditions(x0);
    if (x.op() != ADD) return x;
    std::map<Symbolic, double, AlgebraicHashLess> multiples;
    for (auto& c : mapChildren(x, pullConstant)) multiples[c[1]] += c[0].constant();
    std::vector<Symbolic> childs;
    for (auto& c : multiples) {
        if (c.second != 0.0) {
            if (c.second == 1.0)
                childs.push_back(c.first);
            else
                childs.push_back(flattenMultiplications(Symbolic(c.second) * c.first));
        }
    }
    return makeSymbolic(ADD, childs);
}

// Repeatedly factors out the factor shared by the most summands, weighted by
// its complexity (reference Simplify.cpp:343-417).
Symbolic pullFactor(Symbolic x) {
    if (x.op() != ADD) return x;
    if (x.numChilds() == 1) return x[0];
    if (x.numChilds() == 0) return Symbolic(0.0);
    if (isSmallConstant(x.algebraicHash())) return Symbolic((double)x.algebraicHash());

    std::vector<std::vector<Symbolic>> summands;
    summands.reserve(x.numChilds());
    for (const auto& c : x) {
        if (isMul(c)) {
            std::vector<Symbolic> fs;
            Symbolic fc = flattenMultiplications(c);
            if (fc.op() == MUL) {
                for (auto& cc : flattenMultiplications(c)) fs.push_back(cc);
            } else {
                fs.push_back(fc);
            }
            summands.push_back(std::move(fs));
        } else {
            summands.push_back({c});
        }
    }

    std::map<Symbolic, std::set<int>, AlgebraicHashLess> factors;
    for (int i = 0; i < (int)summands.size(); ++i)
        for (auto& y : summands[i]) factors[y].insert(i);

    auto score = [](const std::pair<const Symbolic, std::set<int>>& a) {
        return std::max((int)a.second.size() - 2, 0) * (a.first.complexity() + 1);
    };
    auto maxIt = std::max_element(factors.begin(), factors.end(),
                                  [&](const auto& a, const auto& b) { return score(a) < score(b); });
    if (maxIt->second.size() < 2) return x;

    auto it = maxIt->second.begin();
    std::vector<Symbolic> factored, rest;
    for (int i = 0; i < (int)summands.size(); ++i) {
        if (it != maxIt->second.end() && i == *it) {
            auto its = std::find(summands[i].begin(), summands[i].end(), maxIt->first);
            summands[i].erase(its);
            if (summands[i].empty())
                factored.push_back(Symbolic(1.0));
            else
                factored.emplace_back(MUL, summands[i]);
            ++it;
        } else {
            rest.emplace_back(MUL, summands[i]);
        }
    }
    rest.push_back(maxIt->first * pullFactor(makeSymbolic(ADD, factored)));
    return pullFactor(flattenAdditions(makeSymbolic(ADD, rest)));
}

namespace {

// Multiplications by -1 become negations; negative summands are grouped under
// one negation (reference Simplify.cpp:419-451).
Symbolic findNegative(const Symbolic& expr) {
    if (expr.op() == MULC && expr[0].constant() == -1) return Symbolic(NEG, expr[1]);
    if (expr.op() == MUL) {
        std::vector<Symbolic> childs;
        int cnt = 0;
        for (auto& c : expr) {
            if (c.op() == CONST && c.constant() == -1.0)
                ++cnt;
            else
                childs.push_back(c);
        }
        if (cnt % 2) return Symbolic(NEG, makeMul(childs));
        return makeMul(childs);
    }
    if (expr.op() == ADD) {
        std::vector<Symbolic> positive, negative;
        for (auto& c : expr) {
            if (c.op() == NEG)
                negative.push_back(c[0]);
            else if (c.op() == MULC && c[0].constant() == -1.0)
                negative.push_back(c[1]);
            else
                positive.push_back(c);
        }
        if (!negative.empty()) positive.emplace_back(NEG, makeAddition(negative));
        return makeAddition(positive);
    }
    return expr;
}

Symbolic simplifyExpression(const Symbolic& expr) {
    if (isSmallConstant(expr.ahash())) return Symbolic((double)expr.ahash());
    if (expr.numChilds() == 0) return expr;
    Symbolic x = optimizeSum(expr);
    x = pullFactor(x);
    x = optimizeProducts(x);
    return x;
}

Symbolic rebuild(const Symbolic& x, const std::vector<Symbolic>& childs) {
    if (x.numChilds() == 0) return x;
    return makeSymbolic(x.op(), childs);
}

}  // namespace

Symbolic simplify(const Symbolic& expr) {
    return traverseGenerate<Symbolic>(
        expr, [](const Symbolic& x) { return simplifyExpression(x); },
        [](const Symbolic& x, const std::vector<Symbolic>& childs) {
            if (x.numChilds() == 0) return x;
            return findNegative(simplifyExpression(makeSymbolic(x.op(), childs)));
        },
        true);
}

// Rebuilds every node through makeSymbolic, memoised by algebraic hash; this
// folds constants and merges algebraically equal sub-trees into one node
// (reference Simplify.cpp:479-505).
Symbolic removeConstantExpressions(const Symbolic& x) {
    return traverseGenerate<Symbolic>(x, [](const Symbolic& y) { return y; }, rebuild, true);
}

Symbolic referenceRedundant(const Symbolic& x) {
    return traverseGenerate<Symbolic>(x, [](const Symbolic& y) { return y; }, rebuild, true);
}

}  // namespace symgb
