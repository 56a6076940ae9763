// Stand-in for Reffine's Z3Solver (include/reffine/pass/z3solver.h; the original wraps the Z3 SMT
// solver, which is not available here).  Used only to build Reffine's own compile path as a test
// oracle.
//
// Reffine asks the solver one kind of question, from Reffine::extract_bound
// (src/pass/reffinepass.cpp:9-53): for one comparison `pred` in an Op's predicate, is there a bias
// b and one weight w_v per variable v (the Func's scalar inputs and the outer iterators) with
//     forall iter, vars:  (iter >= b + sum_v w_v * v) == pred        (a lower bound), or
//     forall iter, vars:  (iter <= b + sum_v w_v * v) == pred        (an upper bound)?
// and, if so, what are b and the w_v (Z3Solver::get on each symbol).
//
// Over the integers (Z3's integer sort: no wrap-around), with pred of the form
// `iter CMP c + sum_v k_v * v` (CMP one of < <= > >=, the iterator alone on either side,
// integer constants c and k_v), the answer is exact and unique:
//     iter >= e  -> lower bound, b = c        iter > e  -> lower bound, b = c + 1
//     iter <= e  -> upper bound, b = c        iter < e  -> upper bound, b = c - 1
// with w_v = k_v, and the opposite query has no solution.  A comparison that does not mention the
// iterator has no solution either: the left side changes with iter, the right side does not.
// Symbols are told apart by name, as Z3 does (Z3Solver::Visit(SymNode&) makes int_const(name)):
// LoopGen quantifies over the cloned Func's inputs while the predicate still names the original
// ones.  Anything outside this fragment (a non-integer iterator, a non-linear term, a symbol that
// is not a quantified variable) throws, so a query the stand-in cannot decide fails instead of
// lowering differently from Reffine.
#ifndef ORACLE_REF_SHIM_Z3SOLVER_H_
#define ORACLE_REF_SHIM_Z3SOLVER_H_

#include <cmath>
#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "reffine/ir/expr.h"

namespace reffine {

class Z3Solver {
public:
    bool check(Expr prop)
    {
        _model.clear();
        auto fa = std::dynamic_pointer_cast<NaryExpr>(prop);
        if (!fa || fa->op != MathOp::FORALL || fa->args.size() < 2) fail("not a forall query");
        std::vector<std::string> vars;
        for (size_t i = 0; i + 1 < fa->args.size(); i++) vars.push_back(name_of(fa->args[i]));
        const std::string iter = vars[0];
        if (iter.empty()) fail("quantified term is not a symbol");
        if (!fa->args[0]->type.is_int() && !fa->args[0]->type.is_idx()) fail("iterator is not an integer");

        auto eq = std::dynamic_pointer_cast<NaryExpr>(fa->args.back());
        if (!eq || eq->op != MathOp::EQ) fail("body is not an equivalence");
        auto lhs = std::dynamic_pointer_cast<NaryExpr>(eq->args[0]);
        auto pred = std::dynamic_pointer_cast<NaryExpr>(eq->args[1]);
        if (!lhs || (lhs->op != MathOp::GTE && lhs->op != MathOp::LTE) || name_of(lhs->args[0]) != iter)
            fail("left side is not a bound of the iterator");
        bool lower = lhs->op == MathOp::GTE;

        // the bound b + sum w_v * v, built as add(mul(w, v), add(..., b))
        Expr bias;
        std::map<std::string, Expr> weight_of;
        Expr cur = lhs->args[1];
        while (true) {
            auto add = std::dynamic_pointer_cast<NaryExpr>(cur);
            if (!add || add->op != MathOp::ADD) break;
            auto mul = std::dynamic_pointer_cast<NaryExpr>(add->args[0]);
            if (!mul || mul->op != MathOp::MUL) fail("bound term is not weight * variable");
            weight_of[name_of(mul->args[1])] = mul->args[0];
            cur = add->args[1];
        }
        if (!std::dynamic_pointer_cast<SymNode>(cur)) fail("bound has no bias symbol");
        bias = cur;

        if (!pred) fail("predicate is not a comparison");
        MathOp op = pred->op;
        if (op != MathOp::LT && op != MathOp::LTE && op != MathOp::GT && op != MathOp::GTE)
            fail("predicate is not an ordering comparison");
        bool iter_left = name_of(pred->args[0]) == iter && !mentions(pred->args[1], iter);
        bool iter_right = name_of(pred->args[1]) == iter && !mentions(pred->args[0], iter);
        if (!iter_left && !iter_right) {
            if (!mentions(pred->args[0], iter) && !mentions(pred->args[1], iter)) return false;
            fail("iterator is not alone on one side");
        }
        if (iter_right) op = flip(op);
        Lin e = linear(iter_left ? pred->args[1] : pred->args[0], vars);

        int64_t b;
        if (lower && op == MathOp::GTE) b = e.c;
        else if (lower && op == MathOp::GT) b = e.c + 1;
        else if (!lower && op == MathOp::LTE) b = e.c;
        else if (!lower && op == MathOp::LT) b = e.c - 1;
        else return false;

        _model[bias.get()] = std::make_shared<Const>(bias->type, (double)b);
        for (auto& [v, w] : weight_of) {
            auto it = e.k.find(v);
            int64_t k = it == e.k.end() ? 0 : it->second;
            _model[w.get()] = std::make_shared<Const>(w->type, (double)k);
        }
        return true;
    }

    shared_ptr<Const> get(Expr sym)
    {
        auto it = _model.find(sym.get());
        if (it == _model.end()) fail("symbol has no value in the model");
        return it->second;
    }

private:
    struct Lin {
        int64_t c = 0;
        std::map<std::string, int64_t> k;
    };

    [[noreturn]] static void fail(const std::string& why)
    {
        throw std::runtime_error("Z3 stand-in: query outside its fragment (" + why + ")");
    }

    static MathOp flip(MathOp op)
    {
        switch (op) {
            case MathOp::LT: return MathOp::GT;
            case MathOp::LTE: return MathOp::GTE;
            case MathOp::GT: return MathOp::LT;
            default: return MathOp::LTE;
        }
    }

    static std::string name_of(const Expr& e)
    {
        auto s = std::dynamic_pointer_cast<SymNode>(e);
        return s ? s->name : std::string();
    }

    static bool mentions(const Expr& e, const std::string& s)
    {
        if (std::dynamic_pointer_cast<SymNode>(e)) return name_of(e) == s;
        if (std::dynamic_pointer_cast<Const>(e)) return false;
        if (auto n = std::dynamic_pointer_cast<NaryExpr>(e)) {
            for (auto& a : n->args)
                if (mentions(a, s)) return true;
            return false;
        }
        if (auto c = std::dynamic_pointer_cast<Cast>(e)) return mentions(c->arg, s);
        fail("cannot look inside a term");
    }

    static int64_t int_const(const Expr& e)
    {
        auto c = std::dynamic_pointer_cast<Const>(e);
        if (!c || !(c->type.is_int() || c->type.is_idx())) fail("non-integer constant");
        return (int64_t)c->val;
    }

    static Lin linear(const Expr& e, const std::vector<std::string>& vars)
    {
        Lin r;
        if (auto c = std::dynamic_pointer_cast<Const>(e)) {
            r.c = int_const(e);
            return r;
        }
        if (std::dynamic_pointer_cast<SymNode>(e)) {
            for (size_t i = 1; i < vars.size(); i++)
                if (vars[i] == name_of(e)) {
                    r.k[vars[i]] = 1;
                    return r;
                }
            fail("symbol is not a quantified variable");
        }
        auto n = std::dynamic_pointer_cast<NaryExpr>(e);
        if (!n) fail("non-linear term");
        if (n->op == MathOp::ADD || n->op == MathOp::SUB) {
            Lin a = linear(n->args[0], vars), b = linear(n->args[1], vars);
            int64_t s = n->op == MathOp::ADD ? 1 : -1;
            a.c += s * b.c;
            for (auto& [v, k] : b.k) a.k[v] += s * k;
            return a;
        }
        if (n->op == MathOp::NEG) {
            Lin a = linear(n->args[0], vars);
            a.c = -a.c;
            for (auto& kv : a.k) kv.second = -kv.second;
            return a;
        }
        if (n->op == MathOp::MUL) {
            bool lc = (bool)std::dynamic_pointer_cast<Const>(n->args[0]);
            bool rc = (bool)std::dynamic_pointer_cast<Const>(n->args[1]);
            if (!lc && !rc) fail("product of two variables");
            int64_t m = int_const(lc ? n->args[0] : n->args[1]);
            Lin a = linear(lc ? n->args[1] : n->args[0], vars);
            a.c *= m;
            for (auto& kv : a.k) kv.second *= m;
            return a;
        }
        fail("non-linear operator");
    }

    std::map<const ExprNode*, shared_ptr<Const>> _model;
};

}  // namespace reffine

#endif  // ORACLE_REF_SHIM_Z3SOLVER_H_
