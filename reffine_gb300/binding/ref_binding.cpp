// func_text: a reffine::Func, built with Reffine's own builder (include/reffine/builder/reffiner.h
// and the node types of include/reffine/ir/{node,expr,op,op_to_loop,stmt}.h), printed in the text
// form the GPU backend's rf_plan_compile reads.  Compiled as part of a program that includes
// Reffine's headers; the backend itself does not need them.
//
// The text form: (func NAME OUTPUT (inputs (SYM TYPE)...) (tbl (SYM EXPR)...)), expressions as
// S-expressions named after the node kinds (const, add/sub/... by MathOp, sel, cast, get, new,
// op, elem, in, reduce, subvec, len, locate, readdata); types as i8..u64, f32, f64, bool, idx,
// (struct ...), (vector DIM (TYPES) (ENCODINGS)).
#include <cctype>
#include <cmath>
#include <cstdio>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "reffine/base/type.h"
#include "reffine/ir/expr.h"
#include "reffine/ir/node.h"
#include "reffine/ir/op.h"
#include "reffine/ir/op_to_loop.h"
#include "reffine/ir/stmt.h"
#include "reffine_gb300/ref_binding.h"

namespace reffine_gb300 {
namespace {

using reffine::DataType;
using reffine::Expr;
using reffine::Sym;

std::string type_text(const DataType& t)
{
    switch (t.btype) {
        case reffine::VOID: return "void";
        case reffine::BOOL: return "bool";
        case reffine::INT8: return "i8";
        case reffine::INT16: return "i16";
        case reffine::INT32: return "i32";
        case reffine::INT64: return "i64";
        case reffine::UINT8: return "u8";
        case reffine::UINT16: return "u16";
        case reffine::UINT32: return "u32";
        case reffine::UINT64: return "u64";
        case reffine::FLOAT32: return "f32";
        case reffine::FLOAT64: return "f64";
        case reffine::IDX: return "idx";
        case reffine::STRUCT: {
            std::string s = "(struct";
            for (auto& d : t.dtypes) s += " " + type_text(d);
            return s + ")";
        }
        case reffine::VECTOR: {
            std::string s = "(vector " + std::to_string(t.dim) + " (";
            for (size_t i = 0; i < t.dtypes.size(); i++) s += (i ? " " : "") + type_text(t.dtypes[i]);
            s += ") (";
            for (size_t i = 0; i < t.encodings.size(); i++)
                s += std::string(i ? " " : "") + (t.encodings[i] == reffine::RUNEND ? "runend" : "flat");
            return s + "))";
        }
        default: throw std::runtime_error("reffine_gb300: a type the GPU backend does not take");
    }
}

const char* op_text(reffine::MathOp op)
{
    using M = reffine::MathOp;
    switch (op) {
        case M::ADD: return "add";
        case M::SUB: return "sub";
        case M::MUL: return "mul";
        case M::DIV: return "div";
        case M::MAX: return "max";
        case M::MIN: return "min";
        case M::MOD: return "mod";
        case M::SQRT: return "sqrt";
        case M::POW: return "pow";
        case M::ABS: return "abs";
        case M::NEG: return "neg";
        case M::CEIL: return "ceil";
        case M::FLOOR: return "floor";
        case M::LT: return "lt";
        case M::LTE: return "lte";
        case M::GT: return "gt";
        case M::GTE: return "gte";
        case M::EQ: return "eq";
        case M::NOT: return "not";
        case M::AND: return "and";
        case M::OR: return "or";
        default: throw std::runtime_error("reffine_gb300: an operator the GPU backend does not take");
    }
}

std::string num_text(double v)
{
    if (std::isnan(v)) return "nan";
    if (std::isinf(v)) return v > 0 ? "inf" : "-inf";
    char buf[64];
    snprintf(buf, sizeof buf, "%.17g", v);  // round-trips every double
    return buf;
}

class TextPrinter {
public:
    explicit TextPrinter(const reffine::Func& fn) : fn_(fn) {}

    std::string run()
    {
        for (auto& s : fn_.inputs) name(s.get());
        for (auto& kv : fn_.tbl) name(kv.first.get());
        std::ostringstream o;
        const std::string out = e(fn_.output);
        o << "(func " << fn_.name << " " << out << " (inputs";
        for (auto& s : fn_.inputs) o << " (" << name(s.get()) << " " << type_text(s->type) << ")";
        o << ") (tbl";
        for (auto& kv : fn_.tbl) o << " (" << name(kv.first.get()) << " " << e(kv.second) << ")";
        o << "))";
        return o.str();
    }

private:
    // symbol names: the Sym's own name (characters outside [A-Za-z0-9_.$] become '_'), made
    // unique with "#n" where two symbols share a name
    std::string name(const reffine::SymNode* s)
    {
        auto it = names_.find(s);
        if (it != names_.end()) return it->second;
        std::string base;
        for (char c : s->name) base += (isalnum((unsigned char)c) || c == '_' || c == '.' || c == '$') ? c : '_';
        if (base.empty()) base = "sym";
        std::string nm = base;
        for (int i = 1; used_.count(nm); i++) nm = base + "#" + std::to_string(i);
        used_[nm] = 1;
        names_[s] = nm;
        return nm;
    }

    template <class N>
    static const N* is(const Expr& x)
    {
        return dynamic_cast<const N*>(x.get());
    }

    std::string e(const Expr& x)
    {
        if (!x) throw std::runtime_error("reffine_gb300: null expression");
        if (auto s = is<reffine::SymNode>(x)) return name(s);
        if (auto c = is<reffine::Const>(x)) return "(const " + type_text(c->type) + " " + num_text(c->val) + ")";
        if (auto n = is<reffine::NaryExpr>(x)) {
            std::string s = std::string("(") + op_text(n->op);
            for (auto& a : n->args) s += " " + e(a);
            return s + ")";
        }
        if (auto n = is<reffine::Select>(x)) return "(sel " + e(n->cond) + " " + e(n->true_body) + " " + e(n->false_body) + ")";
        if (auto n = is<reffine::Cast>(x)) return "(cast " + type_text(n->type) + " " + e(n->arg) + ")";
        if (auto n = is<reffine::Get>(x)) return "(get " + e(n->val) + " " + std::to_string(n->col) + ")";
        if (auto n = is<reffine::New>(x)) {
            std::string s = "(new";
            for (auto& v : n->vals) s += " " + e(v);
            return s + ")";
        }
        if (auto n = is<reffine::Op>(x)) {
            std::string s = "(op (";
            for (size_t i = 0; i < n->iters.size(); i++)
                s += (i ? " (" : "(") + name(n->iters[i].get()) + " " + type_text(n->iters[i]->type) + ")";
            s += ") " + e(n->pred) + " (";
            for (size_t i = 0; i < n->outputs.size(); i++) s += (i ? " " : "") + e(n->outputs[i]);
            return s + "))";
        }
        if (auto n = is<reffine::Element>(x)) return "(elem " + e(n->vec) + " " + e(n->iter) + ")";
        if (auto n = is<reffine::In>(x)) return "(in " + e(n->iter) + " " + e(n->vec) + ")";
        if (auto n = is<reffine::Reduce>(x)) {
            // op.h:97-112 keeps init and acc as functions: applied once to fresh symbols here
            // (once per node: a Reduce reached twice prints the same text)
            auto done = reduce_text_.find(n);
            if (done != reduce_text_.end()) return done->second;
            auto state = std::make_shared<reffine::SymNode>("state", n->type);
            auto val = std::make_shared<reffine::SymNode>("val", n->vec->type.rowty());
            held_.push_back(state);
            held_.push_back(val);
            Expr init = n->init();
            Expr acc = n->acc(state, val);
            std::string t = "(reduce " + e(n->vec) + " " + e(init) + " (" + name(state.get()) + " " +
                            type_text(state->type) + ") (" + name(val.get()) + " " + type_text(val->type) + ") " + e(acc) +
                            ")";
            reduce_text_[n] = t;
            return t;
        }
        if (auto n = is<reffine::SubVector>(x)) return "(subvec " + e(n->vec) + " " + e(n->start) + " " + e(n->end) + ")";
        if (auto n = is<reffine::Length>(x)) return "(len " + e(n->vec) + " " + std::to_string(n->col) + ")";
        if (auto n = is<reffine::Locate>(x)) {
            // the Call's arguments hold (vec, iter) (op_to_loop.h:106-119)
            if (n->args.size() != 2) throw std::runtime_error("reffine_gb300: malformed Locate");
            return "(locate " + e(n->args[0]) + " " + e(n->args[1]) + ")";
        }
        if (auto n = is<reffine::ReadData>(x))
            return "(readdata " + e(n->vec) + " " + e(n->idx) + " " + std::to_string(n->col) + ")";
        throw std::runtime_error("reffine_gb300: an IR node the GPU backend does not take");
    }

    const reffine::Func& fn_;
    std::unordered_map<const void*, std::string> names_;
    std::map<std::string, int> used_;
    std::vector<Sym> held_;  // fresh symbols stay alive while their addresses key names_
    std::unordered_map<const void*, std::string> reduce_text_;
};

}  // namespace

std::string func_text(const reffine::Func& fn) { return TextPrinter(fn).run(); }

}  // namespace reffine_gb300
