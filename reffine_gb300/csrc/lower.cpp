// Lowering pass: Reffine Func -> kernel template + device fragment (CUDA source).
//
// Reference semantics restated here (Reffine, file:line):
//   iteration spaces   src/pass/reffinepass.cpp:55-123, src/iter/iter_space.cpp (VecSpace,
//                      LBound/UBound/Filtered, the & composition at :6-12)
//   Reduce             src/pass/loopgen.cpp:206-269: row loop over a SubVector (condition:
//                      validity of column 1) or over an Op's iteration space; the accumulator
//                      is applied in row order
//   struct state       src/pass/scalarpass.cpp:121-137 (field-by-field stores)
//   constants          src/pass/cemitter.cpp:89-107 (FP constants printed with 6 decimals)
//   expressions        src/pass/cemitter.cpp:112-160 (C++ operators and std::max/std::min)
#include "lower.h"

#include <algorithm>
#include <array>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <set>
#include <sstream>

namespace rfg {

using namespace reffine;

namespace {

// ------------------------------------------------------------------------------------------
// IR utilities
// ------------------------------------------------------------------------------------------
template <class T>
const T* as(const Expr& e)
{
    return static_cast<const T*>(e.get());
}

bool is_kind(const Expr& e, NodeKind k) { return e && e->kind == k; }

bool is_nary(const Expr& e, MathOp op) { return is_kind(e, NodeKind::NARY) && as<NaryExpr>(e)->op == op; }

// structural equality (symbols by identity)
bool same(const Expr& a, const Expr& b)
{
    if (a.get() == b.get()) return true;
    if (!a || !b || a->kind != b->kind || a->type != b->type) return false;
    switch (a->kind) {
        case NodeKind::SYM: return false;
        case NodeKind::CONST: return as<Const>(a)->val == as<Const>(b)->val;
        case NodeKind::NARY: {
            auto x = as<NaryExpr>(a), y = as<NaryExpr>(b);
            if (x->op != y->op || x->args.size() != y->args.size()) return false;
            for (size_t i = 0; i < x->args.size(); i++)
                if (!same(x->args[i], y->args[i])) return false;
            return true;
        }
        case NodeKind::SELECT: {
            auto x = as<Select>(a), y = as<Select>(b);
            return same(x->cond, y->cond) && same(x->true_body, y->true_body) && same(x->false_body, y->false_body);
        }
        case NodeKind::CAST: return same(as<Cast>(a)->arg, as<Cast>(b)->arg);
        case NodeKind::GET: return as<Get>(a)->col == as<Get>(b)->col && same(as<Get>(a)->val, as<Get>(b)->val);
        case NodeKind::NEW: {
            auto x = as<New>(a), y = as<New>(b);
            if (x->vals.size() != y->vals.size()) return false;
            for (size_t i = 0; i < x->vals.size(); i++)
                if (!same(x->vals[i], y->vals[i])) return false;
            return true;
        }
        case NodeKind::ELEMENT: return same(as<Element>(a)->vec, as<Element>(b)->vec) && same(as<Element>(a)->iter, as<Element>(b)->iter);
        case NodeKind::LENGTH: return as<Length>(a)->col == as<Length>(b)->col && same(as<Length>(a)->vec, as<Length>(b)->vec);
        case NodeKind::LOCATE: return same(as<Locate>(a)->vec, as<Locate>(b)->vec) && same(as<Locate>(a)->iter, as<Locate>(b)->iter);
        case NodeKind::READDATA:
            return as<ReadData>(a)->col == as<ReadData>(b)->col && same(as<ReadData>(a)->vec, as<ReadData>(b)->vec) &&
                   same(as<ReadData>(a)->idx, as<ReadData>(b)->idx);
        default: return false;
    }
}

void children(const Expr& e, std::vector<Expr>& out)
{
    switch (e->kind) {
        case NodeKind::NARY: for (auto& a : as<NaryExpr>(e)->args) out.push_back(a); break;
        case NodeKind::SELECT: {
            auto s = as<Select>(e);
            out.push_back(s->cond), out.push_back(s->true_body), out.push_back(s->false_body);
            break;
        }
        case NodeKind::CAST: out.push_back(as<Cast>(e)->arg); break;
        case NodeKind::GET: out.push_back(as<Get>(e)->val); break;
        case NodeKind::NEW: for (auto& v : as<New>(e)->vals) out.push_back(v); break;
        case NodeKind::OP: {
            auto o = as<Op>(e);
            for (auto& i : o->iters) out.push_back(i);
            out.push_back(o->pred);
            for (auto& x : o->outputs) out.push_back(x);
            break;
        }
        case NodeKind::ELEMENT: out.push_back(as<Element>(e)->vec), out.push_back(as<Element>(e)->iter); break;
        case NodeKind::IN: out.push_back(as<In>(e)->iter), out.push_back(as<In>(e)->vec); break;
        case NodeKind::REDUCE: {
            auto r = as<Reduce>(e);
            out.push_back(r->vec), out.push_back(r->init_expr), out.push_back(r->acc_expr);
            break;
        }
        case NodeKind::SUBVECTOR: {
            auto s = as<SubVector>(e);
            out.push_back(s->vec), out.push_back(s->start), out.push_back(s->end);
            break;
        }
        case NodeKind::LENGTH: out.push_back(as<Length>(e)->vec); break;
        case NodeKind::LOCATE: out.push_back(as<Locate>(e)->vec), out.push_back(as<Locate>(e)->iter); break;
        case NodeKind::READDATA: out.push_back(as<ReadData>(e)->vec), out.push_back(as<ReadData>(e)->idx); break;
        default: break;
    }
}

// does `e` (following table symbols through `tbl`) reference a node in `targets`?
bool mentions(const Expr& e, const std::set<const ExprNode*>& targets, const SymTable& tbl,
              std::set<const ExprNode*>& seen)
{
    if (!e) return false;
    if (targets.count(e.get())) return true;
    if (seen.count(e.get())) return false;
    seen.insert(e.get());
    if (e->kind == NodeKind::SYM) {
        auto it = tbl.find(std::static_pointer_cast<SymNode>(e));
        return it != tbl.end() && mentions(it->second, targets, tbl, seen);
    }
    std::vector<Expr> ch;
    children(e, ch);
    for (auto& c : ch)
        if (mentions(c, targets, tbl, seen)) return true;
    return false;
}

bool mentions(const Expr& e, const ExprNode* target, const SymTable& tbl)
{
    std::set<const ExprNode*> t{target}, seen;
    return mentions(e, t, tbl, seen);
}

void flatten_and(const Expr& e, std::vector<Expr>& out)
{
    if (is_nary(e, MathOp::AND)) {
        flatten_and(as<NaryExpr>(e)->args[0], out);
        flatten_and(as<NaryExpr>(e)->args[1], out);
    } else {
        out.push_back(e);
    }
}

std::string hexkey(const std::string& s)
{
    // FNV-1a 64 over the source: a stable cache key
    unsigned long long h = 1469598103934665603ULL;
    for (unsigned char c : s) h = (h ^ c) * 1099511628211ULL;
    char b[32];
    snprintf(b, sizeof b, "%016llx", h);
    return b;
}

std::string ctype(const DataType& t)
{
    switch (t.btype) {
        case BOOL: return "bool";
        case INT8: return "int8_t";
        case UINT8: return "uint8_t";
        case INT16: return "int16_t";
        case UINT16: return "uint16_t";
        case INT32: return "int32_t";
        case UINT32: return "uint32_t";
        case INT64: case IDX: return "int64_t";
        case UINT64: return "uint64_t";
        case FLOAT32: return "float";
        case FLOAT64: return "double";
        default: throw LowerError("no device type for " + t.str());
    }
}

// ------------------------------------------------------------------------------------------
// Values produced by the expression emitter
// ------------------------------------------------------------------------------------------
struct Val {
    enum K { SCALAR, STRUCT, VEC, SUBVEC } k = SCALAR;
    std::string c;
    std::vector<Val> f;
    int slot = -1;
    int input = -1;
    const ExprNode* vnode = nullptr;
    std::string s, e;
    DataType type;
};

// ------------------------------------------------------------------------------------------
// Accumulator leaves of a Reduce state
// ------------------------------------------------------------------------------------------
enum class AggOp { NONE, SUM, MIN, MAX, OR, AND };

struct Leaf {
    std::vector<size_t> path;
    DataType type;
    AggOp op = AggOp::NONE;
    Expr cond;               // null = every row
    Expr value;              // the row's contribution
    bool state_first = true; // std::max(s, e) vs std::max(e, s)
    bool count = false;      // value is the constant 1: accumulate as an integer count
    Expr init;
    // grouping
    std::vector<Expr> filters;
    std::vector<std::pair<Expr, Expr>> keys;  // (key expression, constant)
};

const char* agg_name(AggOp op)
{
    switch (op) {
        case AggOp::SUM: return "sum";
        case AggOp::MIN: return "min";
        case AggOp::MAX: return "max";
        case AggOp::OR: return "or";
        case AggOp::AND: return "and";
        default: return "none";
    }
}

// ------------------------------------------------------------------------------------------
// Iteration space of a single-iterator Op (reffinepass.cpp:55-105 composed by & as in
// iter_space.cpp:6-12): base VecSpace or UniversalSpace, wrapped by LBound/UBound/Filtered.
// ------------------------------------------------------------------------------------------
struct Space {
    bool has_vec = false;
    int vec_input = -1;              // Func input of the iterated vector
    Expr vec_node;                   // the vector expression (In's vec)
    Expr iter;                       // the iterator symbol
    std::vector<Expr> lbs, ubs;      // bound expressions (iter >= lb, iter <= ub)
    std::vector<Expr> filters;       // boolean symbols
    int n_vecs = 0;
    std::vector<std::pair<int, Expr>> vecs;  // every iterated vector (Func input, In's vec)
};

class Lowerer {
public:
    Lowerer(std::shared_ptr<Func> fn, bool vectorize, int threads)
        : fn_(std::move(fn)), vectorize_(vectorize), threads_(threads)
    {
    }

    Plan run()
    {
        plan_.vectorize = vectorize_;
        plan_.threads = threads_;
        plan_.n_inputs = (int)fn_->inputs.size();
        int tslot = 0, sslot = 0;
        for (size_t i = 0; i < fn_->inputs.size(); i++) {
            auto& s = fn_->inputs[i];
            plan_.input_types.push_back(s->type);
            plan_.cols_read.emplace_back();
            plan_.needs_index.push_back(0);
            plan_.random_read.push_back(0);
            if (s->type.is_vector()) {
                if (tslot >= RF_MAX_TABLES_) throw LowerError("too many table inputs");
                if (s->type.dtypes.size() > (size_t)RF_MAX_COLS_) throw LowerError("too many columns");
                plan_.table_slot.push_back(tslot++);
                plan_.scalar_slot.push_back(-1);
            } else if (s->type.is_primitive()) {
                if (sslot >= RF_MAX_SCALARS_) throw LowerError("too many scalar inputs");
                plan_.table_slot.push_back(-1);
                plan_.scalar_slot.push_back(sslot++);
            } else {
                throw LowerError("struct inputs are not supported", false);  // scalarpass.cpp:201-203
            }
            input_index_[s.get()] = (int)i;
        }
        plan_.out_type = fn_->output->type;
        Expr root = resolve(fn_->output);
        if (root->type.is_vector()) {
            if (root->kind != NodeKind::OP) throw LowerError("a vector output must be an Op");
            lower_op(root);
        } else {
            std::vector<const Reduce*> reds;
            find_reduces(fn_->output, reds);
            if (reds.size() != 1) throw LowerError("the GPU backend lowers Funcs with exactly one Reduce");
            lower_reduce(*reds[0]);
        }
        derive_cols_read();
        plan_.key = hexkey(plan_.source);
        return plan_;
    }

    // the columns a plan reads are exactly those its generated source references
    // (P.t[slot].col[c]); table uploads and byte accounting use this set
    void derive_cols_read()
    {
        const std::string& s = plan_.source;
        const std::string pat = "P.t[";
        for (size_t pos = s.find(pat); pos != std::string::npos; pos = s.find(pat, pos + 1)) {
            size_t a = pos + pat.size();
            size_t b = s.find("].col[", a);
            if (b == std::string::npos || b - a > 2) continue;
            size_t c0 = b + 6, c1 = s.find(']', c0);
            if (c1 == std::string::npos || c1 - c0 > 3) continue;
            int slot = std::atoi(s.substr(a, b - a).c_str());
            int col = std::atoi(s.substr(c0, c1 - c0).c_str());
            for (size_t i = 0; i < plan_.table_slot.size(); i++)
                if (plan_.table_slot[i] == slot) note_col((int)i, (size_t)col);
        }
        for (auto& v : plan_.cols_read) std::sort(v.begin(), v.end());
    }

private:
    static constexpr int RF_MAX_TABLES_ = 4, RF_MAX_COLS_ = 24, RF_MAX_SCALARS_ = 16, RF_MAX_CONSTS_ = 128;

    // follow a symbol to its table entry (top-level structure only)
    Expr resolve(const Expr& e) const
    {
        Expr x = e;
        for (int n = 0; n < 64 && x->kind == NodeKind::SYM; n++) {
            auto it = fn_->tbl.find(std::static_pointer_cast<SymNode>(x));
            if (it == fn_->tbl.end()) break;
            x = it->second;
        }
        return x;
    }

    void find_reduces(const Expr& e, std::vector<const Reduce*>& out)
    {
        std::set<const ExprNode*> seen;
        std::function<void(const Expr&)> rec = [&](const Expr& x) {
            if (!x || seen.count(x.get())) return;
            seen.insert(x.get());
            if (x->kind == NodeKind::REDUCE) {
                out.push_back(as<Reduce>(x));
                return;
            }
            if (x->kind == NodeKind::SYM) {
                auto it = fn_->tbl.find(std::static_pointer_cast<SymNode>(x));
                if (it != fn_->tbl.end()) rec(it->second);
                return;
            }
            std::vector<Expr> ch;
            children(x, ch);
            for (auto& c : ch) rec(c);
        };
        rec(e);
    }

    // ---------------------------------------------------------------- constants & inputs
    std::string konst(const Const& c)
    {
        if (c.type.btype == BOOL) return c.val != 0 ? "true" : "false";
        ConstSlot k;
        if (c.type.is_float()) {
            // CEmitter prints FP constants with std::to_string, i.e. "%f" (cemitter.cpp:104-105)
            char buf[512];
            snprintf(buf, sizeof buf, "%f", c.val);
            k.is_float = true;
            k.f = strtod(buf, nullptr);
        } else if (c.type.is_unsigned()) {
            k.i = (long long)(unsigned long long)c.val;
        } else {
            k.i = (long long)c.val;
        }
        // one slot per distinct (kind, value): equal constants read the same slot, so the
        // compiler can share the comparisons that use them
        int i = -1;
        for (size_t j = 0; j < plan_.consts.size(); j++) {
            auto& q = plan_.consts[j];
            if (q.is_float == k.is_float && (k.is_float ? (memcmp(&q.f, &k.f, 8) == 0) : q.i == k.i)) i = (int)j;
        }
        if (i < 0) {
            if (plan_.consts.size() >= (size_t)RF_MAX_CONSTS_) throw LowerError("too many constants");
            i = (int)plan_.consts.size();
            plan_.consts.push_back(k);
        }
        if (c.type.btype == FLOAT64) return "P.k[" + std::to_string(i) + "].f";
        if (c.type.btype == FLOAT32) return "((float)P.k[" + std::to_string(i) + "].f)";
        return "((" + ctype(c.type) + ")P.k[" + std::to_string(i) + "].i)";
    }

    void note_col(int input, size_t col)
    {
        auto& v = plan_.cols_read[input];
        if (std::find(v.begin(), v.end(), (int)col) == v.end()) v.push_back((int)col);
    }

    // ---------------------------------------------------------------- expression emitter
    struct Scope {
        std::map<const ExprNode*, Val> bind;
    };

    struct Emitter {
        Lowerer& L;
        std::vector<Scope> scopes{1};
        std::vector<std::string> decls;  // lazy symbol closures, in dependency order
        std::map<std::pair<const ExprNode*, const ExprNode*>, std::string> vec_iter_idx;
        std::map<std::string, std::string> locate_cache;
        int counter = 0;
        bool in_bounds_rows = true;

        explicit Emitter(Lowerer& l) : L(l) {}

        std::string fresh(const std::string& b) { return b + std::to_string(counter++); }
        void bind(const Expr& s, Val v) { scopes.back().bind[s.get()] = std::move(v); }
        const Val* lookup(const ExprNode* s) const
        {
            for (auto it = scopes.rbegin(); it != scopes.rend(); ++it) {
                auto f = it->bind.find(s);
                if (f != it->bind.end()) return &f->second;
            }
            return nullptr;
        }

        Val scalar(const std::string& c, const DataType& t)
        {
            Val v;
            v.c = c;
            v.type = t;
            return v;
        }

        // a table symbol of primitive type becomes a lazily evaluated, cached closure, so
        // short-circuit conditions keep skipping expensive probes and each value is computed once
        Val lazy(const std::string& base, const Val& v, const DataType& t)
        {
            if (v.k != Val::SCALAR) return v;
            std::string nm = fresh("lz_" + base + "_");
            std::string ty = ctype(t);
            decls.push_back(ty + " " + nm + "_v; bool " + nm + "_h = false; auto " + nm + " = [&]() -> " + ty +
                            " { if (!" + nm + "_h) { " + nm + "_h = true; " + nm + "_v = (" + ty + ")(" + v.c +
                            "); } return " + nm + "_v; };");
            return scalar(nm + "()", t);
        }

        std::map<const ExprNode*, Val> node_bind;  // precomputed values of non-symbol nodes (Reduce)

        Val ev(const Expr& e)
        {
            auto nb = node_bind.find(e.get());
            if (nb != node_bind.end()) return nb->second;
            switch (e->kind) {
                case NodeKind::SYM: {
                    if (auto b = lookup(e.get())) return *b;
                    auto sym = std::static_pointer_cast<SymNode>(e);
                    auto it = L.fn_->tbl.find(sym);
                    if (it == L.fn_->tbl.end()) throw LowerError("unbound symbol " + sym->name, false);
                    Val v = ev(it->second);
                    if (v.k == Val::SCALAR) {
                        std::string base;
                        for (char ch : sym->name) base += isalnum((unsigned char)ch) ? ch : '_';
                        v = lazy(base, v, sym->type);
                    }
                    scopes.front().bind[e.get()] = v;
                    return v;
                }
                case NodeKind::CONST: return scalar(L.konst(*as<Const>(e)), e->type);
                case NodeKind::NARY: return nary(*as<NaryExpr>(e));
                case NodeKind::SELECT: {
                    auto s = as<Select>(e);
                    Val c = ev(s->cond);
                    return sel(c.c, ev(s->true_body), ev(s->false_body));
                }
                case NodeKind::CAST: {
                    auto c = as<Cast>(e);
                    return scalar("((" + ctype(c->type) + ")(" + ev(c->arg).c + "))", c->type);
                }
                case NodeKind::GET: {
                    auto g = as<Get>(e);
                    Val v = ev(g->val);
                    if (v.k == Val::STRUCT) return v.f.at(g->col);
                    return v;
                }
                case NodeKind::NEW: {
                    Val v;
                    v.k = Val::STRUCT;
                    v.type = e->type;
                    for (auto& x : as<New>(e)->vals) v.f.push_back(ev(x));
                    return v;
                }
                case NodeKind::ELEMENT: return element(*as<Element>(e));
                case NodeKind::SUBVECTOR: {
                    auto s = as<SubVector>(e);
                    Val v = ev(s->vec);
                    if (v.k != Val::VEC) throw LowerError("subvector of a non-input vector");
                    Val r;
                    r.k = Val::SUBVEC;
                    r.slot = v.slot;
                    r.input = v.input;
                    r.vnode = v.vnode;
                    r.type = e->type;
                    r.s = ev(s->start).c;
                    r.e = ev(s->end).c;
                    return r;
                }
                case NodeKind::LENGTH: {
                    auto l = as<Length>(e);
                    Val v = ev(l->vec);
                    if (v.k != Val::VEC) throw LowerError("length of a non-input vector");
                    return scalar("P.t[" + std::to_string(v.slot) + "].col[" + std::to_string(l->col) + "].len", e->type);
                }
                case NodeKind::LOCATE: {
                    auto l = as<Locate>(e);
                    Val v = ev(l->vec);
                    if (v.k != Val::VEC) throw LowerError("locate in a non-input vector");
                    return scalar(locate(v, ev(l->iter).c), e->type);
                }
                case NodeKind::READDATA: {
                    auto r = as<ReadData>(e);
                    Val v = ev(r->vec);
                    if (v.k != Val::VEC) throw LowerError("readdata of a non-input vector");
                    L.note_col(v.input, r->col);
                    L.plan_.random_read[v.input] = 1;
                    return scalar("rf_rd<" + ctype(r->type) + ">(P.t[" + std::to_string(v.slot) + "].col[" +
                                      std::to_string(r->col) + "], (long long)(" + ev(r->idx).c + "))",
                                  r->type);
                }
                case NodeKind::IN: throw LowerError("In outside an Op predicate");
                case NodeKind::OP: throw LowerError("a nested Op inside an expression is not lowered");
                case NodeKind::REDUCE: throw LowerError("a Reduce nested inside this expression is not lowered");
            }
            throw LowerError("unknown node");
        }

        std::string locate(const Val& vec, const std::string& key)
        {
            L.plan_.needs_index[vec.input] = 1;
            L.plan_.random_read[vec.input] = 1;
            L.note_col(vec.input, 0);
            std::string call = "rf_locate(P.t[" + std::to_string(vec.slot) + "].ix, (long long)(" + key + "))";
            auto it = locate_cache.find(call);
            if (it != locate_cache.end()) return it->second;
            Val v = lazy("loc", scalar(call, types::IDX_T), types::IDX_T);
            locate_cache[call] = v.c;
            return v.c;
        }

        Val sel(const std::string& c, const Val& a, const Val& b)
        {
            if (a.k == Val::STRUCT) {
                Val v;
                v.k = Val::STRUCT;
                v.type = a.type;
                for (size_t i = 0; i < a.f.size(); i++) v.f.push_back(sel(c, a.f[i], b.f[i]));
                return v;
            }
            return scalar("(" + c + " ? " + a.c + " : " + b.c + ")", a.type);
        }

        Val element(const Element& el)
        {
            Val vec = ev(el.vec);
            if (vec.k != Val::VEC) throw LowerError("element of a non-input vector");
            std::string idx;
            bool inb = false;
            auto key = std::make_pair(el.vec.get(), el.iter.get());
            auto f = vec_iter_idx.find(key);
            if (f != vec_iter_idx.end()) {
                idx = f->second;
                inb = in_bounds_rows;
            } else {
                idx = locate(vec, ev(el.iter).c);
            }
            const DataType& vt = vec.type;
            if (vt.dim == 1) {
                Val v;
                v.k = Val::STRUCT;
                v.type = el.type;
                for (size_t c = vt.dim; c < vt.dtypes.size(); c++) {
                    L.note_col(vec.input, c);
                    std::string col = "P.t[" + std::to_string(vec.slot) + "].col[" + std::to_string(c) + "]";
                    if (inb)
                        v.f.push_back(scalar("rf_ld<" + ctype(vt.dtypes[c]) + ">(" + col + ".data, " + idx + ")", vt.dtypes[c]));
                    else
                        v.f.push_back(scalar("rf_rd<" + ctype(vt.dtypes[c]) + ">(" + col + ", " + idx + ")", vt.dtypes[c]));
                }
                return v;
            }
            if (vt.dim == 2) {
                if (vt.encodings[0] != RUNEND) throw LowerError("a 2-d element needs a run-end encoded column 0");
                Val r;
                r.k = Val::SUBVEC;
                r.slot = vec.slot;
                r.input = vec.input;
                r.vnode = vec.vnode;
                r.type = el.type;
                std::string c0 = "P.t[" + std::to_string(vec.slot) + "].col[0]";
                r.s = "rf_runend(" + c0 + ", (" + idx + ") - 1)";
                r.e = "rf_runend(" + c0 + ", " + idx + ")";
                return r;
            }
            throw LowerError("Only support 1d and 2d vectors");
        }

        Val nary(const NaryExpr& n)
        {
            auto a = [&](size_t i) { return ev(n.args[i]).c; };
            const std::string T = n.type.is_primitive() ? ctype(n.type) : "";
            switch (n.op) {
                case MathOp::ADD: return scalar("(" + a(0) + " + " + a(1) + ")", n.type);
                case MathOp::SUB: return scalar("(" + a(0) + " - " + a(1) + ")", n.type);
                case MathOp::MUL:
                    // x * (1 - y) and x * (1 + y) in binary64 as one fused multiply-add
                    // (rf_mul_1m / rf_mul_1p in rf_device.cuh: one FP64 operation instead of two)
                    if (n.type.btype == FLOAT64)
                        for (size_t s = 0; s < 2; s++) {
                            const Expr& f = n.args[1 - s];
                            const bool sub = is_nary(f, MathOp::SUB), add = is_nary(f, MathOp::ADD);
                            if (!sub && !add) continue;
                            auto fn = as<NaryExpr>(f);
                            if (!is_kind(fn->args[0], NodeKind::CONST) || fn->args[0]->type.btype != FLOAT64 ||
                                fn->args[1]->type.btype != FLOAT64 || as<Const>(fn->args[0])->val != 1.0)
                                continue;
                            return scalar(std::string(sub ? "rf_mul_1m(" : "rf_mul_1p(") + a(s) + ", " +
                                              ev(fn->args[1]).c + ")",
                                          n.type);
                        }
                    return scalar("(" + a(0) + " * " + a(1) + ")", n.type);
                case MathOp::DIV: return scalar("(" + a(0) + " / " + a(1) + ")", n.type);
                case MathOp::MOD: return scalar("(" + a(0) + " % " + a(1) + ")", n.type);
                case MathOp::MAX: return scalar("rf_max<" + T + ">(" + a(0) + ", " + a(1) + ")", n.type);
                case MathOp::MIN: return scalar("rf_min<" + T + ">(" + a(0) + ", " + a(1) + ")", n.type);
                case MathOp::LT: case MathOp::LTE: case MathOp::GT: case MathOp::GTE: case MathOp::EQ: {
                    static const char* sym[] = {"<", "<=", ">", ">=", "=="};
                    static const char* dfn[] = {"rf_dlt", "rf_dle", "rf_dgt", "rf_dge", "rf_deq"};
                    int k = n.op == MathOp::LT ? 0 : n.op == MathOp::LTE ? 1 : n.op == MathOp::GT ? 2 : n.op == MathOp::GTE ? 3 : 4;
                    // binary64 comparisons go to the integer pipe (exact IEEE semantics, rf_device.cuh)
                    if (n.args[0]->type.btype == FLOAT64)
                        return scalar(std::string(dfn[k]) + "(" + a(0) + ", " + a(1) + ")", n.type);
                    return scalar("(" + a(0) + " " + sym[k] + " " + a(1) + ")", n.type);
                }
                case MathOp::NOT: return scalar("(!" + a(0) + ")", n.type);
                case MathOp::AND: return scalar("(" + a(0) + " && " + a(1) + ")", n.type);
                case MathOp::OR: return scalar("(" + a(0) + " || " + a(1) + ")", n.type);
                case MathOp::NEG: return scalar("(-" + a(0) + ")", n.type);
                case MathOp::SQRT: return scalar("sqrt(" + a(0) + ")", n.type);
                case MathOp::CEIL: return scalar("ceil(" + a(0) + ")", n.type);
                case MathOp::FLOOR: return scalar("floor(" + a(0) + ")", n.type);
                case MathOp::POW:
                    // single precision through the double pow, rounded once: within CUDA's documented
                    // double pow error of the host's correctly rounded powf, where powf alone is 2 ulp
                    if (n.type.btype == FLOAT32)
                        return scalar("((float)pow((double)(" + a(0) + "), (double)(" + a(1) + ")))", n.type);
                    return scalar("pow(" + a(0) + ", " + a(1) + ")", n.type);
                case MathOp::ABS:
                    if (n.type.is_float()) return scalar("fabs(" + a(0) + ")", n.type);
                    return scalar("((" + T + ")llabs((long long)(" + a(0) + ")))", n.type);
                default: throw LowerError(std::string("operator not lowered: ") + mathop_name(n.op));
            }
        }
    };

    Val input_val(int i)
    {
        auto& s = fn_->inputs[i];
        Val v;
        v.type = s->type;
        if (s->type.is_vector()) {
            v.k = Val::VEC;
            v.slot = plan_.table_slot[i];
            v.input = i;
            v.vnode = s.get();
        } else {
            int j = plan_.scalar_slot[i];
            if (s->type.is_float())
                v.c = "((" + ctype(s->type) + ")__longlong_as_double(P.s[" + std::to_string(j) + "]))";
            else
                v.c = "((" + ctype(s->type) + ")P.s[" + std::to_string(j) + "])";
        }
        return v;
    }

    void bind_inputs(Emitter& E)
    {
        for (size_t i = 0; i < fn_->inputs.size(); i++) E.bind(fn_->inputs[i], input_val((int)i));
    }

    // host-evaluable expression (loop bounds)
    HostExpr host_expr(const Expr& e0)
    {
        Expr e = resolve(e0);
        HostExpr h;
        switch (e->kind) {
            case NodeKind::CONST:
                h.kind = HostExpr::CONST;
                h.value = (long long)as<Const>(e)->val;
                return h;
            case NodeKind::LENGTH: {
                auto l = as<Length>(e);
                auto it = input_index_.find(resolve(l->vec).get());
                if (it == input_index_.end()) throw LowerError("loop bound: length of a non-input vector");
                h.kind = HostExpr::LEN;
                h.input = it->second;
                h.col = (int)l->col;
                return h;
            }
            case NodeKind::SYM: {
                auto it = input_index_.find(e.get());
                if (it == input_index_.end() || !e->type.is_primitive()) throw LowerError("loop bound: unknown symbol");
                h.kind = HostExpr::SCALAR;
                h.input = it->second;
                return h;
            }
            case NodeKind::CAST: return host_expr(as<Cast>(e)->arg);
            case NodeKind::NARY: {
                auto n = as<NaryExpr>(e);
                switch (n->op) {
                    case MathOp::ADD: h.kind = HostExpr::ADD; break;
                    case MathOp::SUB: h.kind = HostExpr::SUB; break;
                    case MathOp::MUL: h.kind = HostExpr::MUL; break;
                    case MathOp::MAX: h.kind = HostExpr::MAX; break;
                    case MathOp::MIN: h.kind = HostExpr::MIN; break;
                    default: throw LowerError("loop bound: operator not evaluable on the host");
                }
                for (auto& a : n->args) h.args.push_back(host_expr(a));
                return h;
            }
            default: throw LowerError("loop bound not evaluable on the host");
        }
    }

    // ---------------------------------------------------------------- iteration space
    bool affine(const Expr& e, const std::set<const ExprNode*>& vars)
    {
        switch (e->kind) {
            case NodeKind::CONST: return true;
            case NodeKind::SYM: return vars.count(e.get()) > 0;
            case NodeKind::NARY: {
                auto n = as<NaryExpr>(e);
                if (n->op == MathOp::ADD || n->op == MathOp::SUB) return affine(n->args[0], vars) && affine(n->args[1], vars);
                if (n->op == MathOp::NEG) return affine(n->args[0], vars);
                if (n->op == MathOp::MUL)
                    return (is_kind(n->args[0], NodeKind::CONST) && affine(n->args[1], vars)) ||
                           (is_kind(n->args[1], NodeKind::CONST) && affine(n->args[0], vars));
                return false;
            }
            default: return false;
        }
    }

    // Reffine::visit + Reffine::extract_bound restated for `iter <op> affine(vars)`
    void space_of(const Expr& pred, const Expr& iter, const std::set<const ExprNode*>& vars, Space& sp)
    {
        if (is_nary(pred, MathOp::AND)) {
            space_of(as<NaryExpr>(pred)->args[0], iter, vars, sp);
            space_of(as<NaryExpr>(pred)->args[1], iter, vars, sp);
            return;
        }
        if (pred->kind == NodeKind::NARY) {
            auto n = as<NaryExpr>(pred);
            if (n->op == MathOp::OR) throw LowerError("union iteration spaces are not lowered");
            if (n->op == MathOp::LT || n->op == MathOp::LTE || n->op == MathOp::GT || n->op == MathOp::GTE) {
                Expr a = n->args[0], b = n->args[1];
                MathOp op = n->op;
                Expr rhs;
                if (a.get() == iter.get() && !mentions(b, iter.get(), fn_->tbl)) {
                    rhs = b;
                } else if (b.get() == iter.get() && !mentions(a, iter.get(), fn_->tbl)) {
                    rhs = a;
                    op = op == MathOp::LT ? MathOp::GT : op == MathOp::LTE ? MathOp::GTE : op == MathOp::GT ? MathOp::LT : MathOp::LTE;
                } else if (!mentions(pred, iter.get(), fn_->tbl)) {
                    return;  // no bound solves the forall query: universal space, predicate dropped
                } else {
                    throw LowerError("iterator bound form not lowered");
                }
                if (!affine(rhs, vars) || !(iter->type.is_int() || iter->type.is_idx())) return;  // universal
                auto one = std::make_shared<Const>(iter->type, 1.0);
                if (op == MathOp::GTE) sp.lbs.push_back(rhs);
                else if (op == MathOp::GT) sp.lbs.push_back(reffiner::_add(rhs, one));
                else if (op == MathOp::LTE) sp.ubs.push_back(rhs);
                else sp.ubs.push_back(reffiner::_sub(rhs, one));
                return;
            }
            throw LowerError(std::string("Operator not supported by Reffine: ") + mathop_name(n->op));
        }
        if (pred->kind == NodeKind::SYM) {
            if (pred.get() == iter.get()) return;
            auto it = fn_->tbl.find(std::static_pointer_cast<SymNode>(pred));
            if (it == fn_->tbl.end()) throw LowerError("Unable to reffine symbol");
            if (pred->type == types::BOOL_T) {
                sp.filters.push_back(pred);
                return;
            }
            space_of(it->second, iter, vars, sp);
            return;
        }
        if (pred->kind == NodeKind::IN) {
            auto in = as<In>(pred);
            if (in->iter.get() != iter.get()) throw LowerError("In over another iterator");
            Expr vec = resolve(in->vec);
            auto f = input_index_.find(vec.get());
            if (f == input_index_.end()) throw LowerError("iteration over a non-input vector");
            sp.n_vecs++;
            sp.vecs.push_back({f->second, in->vec});
            if (!sp.has_vec) {
                sp.has_vec = true;
                sp.vec_input = f->second;
                sp.vec_node = in->vec;
            }
            return;
        }
        throw LowerError("predicate node not lowered");
    }

    Space op_space(const Op& op)
    {
        if (op.iters.size() != 1) throw LowerError("multi-iterator Op");
        Space sp;
        sp.iter = op.iters[0];
        std::set<const ExprNode*> vars;
        for (auto& s : fn_->inputs)
            if (s->type.is_val()) vars.insert(s.get());
        space_of(op.pred, sp.iter, vars, sp);
        if (!sp.has_vec && sp.lbs.empty()) throw LowerError("unbounded iteration space (no lower bound)");
        if (!sp.has_vec && sp.ubs.empty()) throw LowerError("unbounded iteration space (no upper bound)");
        return sp;
    }

    // combine bounds as the LBound/UBound chain does: L = max(lbs..., base lb), U = min(ubs..., base ub)
    std::string bound_expr(Emitter& E, const std::vector<Expr>& bs, const std::string& base, bool is_max,
                           const DataType& t)
    {
        std::string r = base;
        for (auto& b : bs) {
            std::string c = "((" + ctype(t) + ")(" + E.ev(b).c + "))";
            r = r.empty() ? c : (std::string(is_max ? "rf_max<" : "rf_min<") + ctype(t) + ">(" + c + ", " + r + ")");
        }
        return r;
    }

    // ---------------------------------------------------------------- Reduce analysis
    std::map<std::vector<size_t>, Expr> leaf_syms_;
    std::map<const ExprNode*, std::vector<size_t>> leaf_path_;

    Expr leaf_sym(const std::vector<size_t>& path, const DataType& t)
    {
        auto it = leaf_syms_.find(path);
        if (it != leaf_syms_.end()) return it->second;
        std::string nm = "$state";
        for (auto p : path) nm += "." + std::to_string(p);
        auto s = std::make_shared<SymNode>(nm, t);
        leaf_syms_[path] = s;
        leaf_path_[s.get()] = path;
        return s;
    }

    // Get(...(state)...) chains become leaf symbols; Get(New)/Get(Select) are simplified
    // does e (through the symbol table) reach the reduce's state?  Memoised per node: simplify
    // asks it of every node it visits, and the accumulator expressions share subtrees.  The
    // cache holds each node, so no address is reused while it is cached.
    std::map<std::pair<const ExprNode*, const ExprNode*>, std::pair<Expr, bool>> mentions_memo_;

    bool mentions_red(const Expr& e, const Reduce& red)
    {
        auto k = std::make_pair(e.get(), (const ExprNode*)red.state.get());
        auto it = mentions_memo_.find(k);
        if (it != mentions_memo_.end()) return it->second.second;
        bool v = mentions(e, red.state.get(), fn_->tbl);
        mentions_memo_.emplace(k, std::make_pair(e, v));
        return v;
    }

    std::map<std::pair<const ExprNode*, const ExprNode*>, std::pair<Expr, Expr>> simplify_memo_;

    // simplify, memoised per node (the accumulator expressions share subtrees); the cache
    // holds each node so no address is reused while cached
    Expr simplify(const Expr& e, const Reduce& red)
    {
        auto k = std::make_pair(e.get(), (const ExprNode*)red.state.get());
        auto it = simplify_memo_.find(k);
        if (it != simplify_memo_.end()) return it->second.second;
        Expr r = simplify_node(e, red);
        simplify_memo_.emplace(k, std::make_pair(e, r));
        return r;
    }

    Expr simplify_node(const Expr& e, const Reduce& red)
    {
        if (e.get() == red.state.get()) {
            if (red.state->type.is_struct()) return e;
            return leaf_sym({}, red.state->type);
        }
        switch (e->kind) {
            case NodeKind::GET: {
                auto g = as<Get>(e);
                Expr v = simplify(g->val, red);
                if (v.get() == red.state.get()) return leaf_sym({g->col}, e->type);
                auto lp = leaf_path_.find(v.get());
                if (lp != leaf_path_.end() && v->type.is_struct()) {
                    auto p = lp->second;
                    p.push_back(g->col);
                    return leaf_sym(p, e->type);
                }
                if (v->kind == NodeKind::NEW) return simplify(as<New>(v)->vals.at(g->col), red);
                if (v->kind == NodeKind::SELECT) {
                    auto s = as<Select>(v);
                    return std::make_shared<Select>(s->cond, simplify(std::make_shared<Get>(s->true_body, g->col), red),
                                                    simplify(std::make_shared<Get>(s->false_body, g->col), red));
                }
                if (v->kind == NodeKind::SYM && v->type.is_struct()) {
                    auto it = fn_->tbl.find(std::static_pointer_cast<SymNode>(v));
                    if (it != fn_->tbl.end() && mentions_red(it->second, red))
                        return simplify(std::make_shared<Get>(it->second, g->col), red);
                }
                if (v.get() == g->val.get()) return e;
                return std::make_shared<Get>(v, g->col);
            }
            case NodeKind::SELECT: {
                auto s = as<Select>(e);
                if (!mentions_red(e, red)) return e;
                return std::make_shared<Select>(simplify(s->cond, red), simplify(s->true_body, red),
                                                simplify(s->false_body, red));
            }
            case NodeKind::NARY: {
                auto n = as<NaryExpr>(e);
                if (!mentions_red(e, red)) return e;
                std::vector<Expr> args;
                for (auto& a : n->args) args.push_back(simplify(a, red));
                return std::make_shared<NaryExpr>(n->type, n->op, args);
            }
            case NodeKind::NEW: {
                if (!mentions_red(e, red)) return e;
                std::vector<Expr> v;
                for (auto& x : as<New>(e)->vals) v.push_back(simplify(x, red));
                return std::make_shared<New>(v);
            }
            case NodeKind::CAST: {
                if (!mentions_red(e, red)) return e;
                return std::make_shared<Cast>(e->type, simplify(as<Cast>(e)->arg, red));
            }
            case NodeKind::SYM: {
                if (e->type.is_struct() || !mentions_red(e, red)) return e;
                auto it = fn_->tbl.find(std::static_pointer_cast<SymNode>(e));
                if (it != fn_->tbl.end()) return simplify(it->second, red);
                return e;
            }
            default: return e;
        }
    }

    Expr field(const Expr& e, const std::vector<size_t>& path, const Reduce& red)
    {
        Expr x = e;
        for (auto p : path) x = simplify(std::make_shared<Get>(x, p), red);
        return simplify(x, red);
    }

    bool mentions_state(const Expr& e)
    {
        std::set<const ExprNode*> t, seen;
        for (auto& kv : leaf_syms_) t.insert(kv.second.get());
        return mentions(e, t, fn_->tbl, seen);
    }

    void collect_leaves(const Reduce& red, const DataType& t, std::vector<size_t> path, std::vector<Leaf>& out)
    {
        if (t.is_struct()) {
            for (size_t i = 0; i < t.dtypes.size(); i++) {
                auto p = path;
                p.push_back(i);
                collect_leaves(red, t.dtypes[i], p, out);
            }
            return;
        }
        if (!t.is_primitive()) throw LowerError("reduce state must be primitives and structs");
        Leaf lf;
        lf.path = path;
        lf.type = t;
        Expr ls = leaf_sym(path, t);
        Expr E = field(red.acc_expr, path, red);
        lf.init = path.empty() ? red.init_expr : field(red.init_expr, path, red);
        // peel conditional updates: sel(c, update, s) / sel(c, s, update)
        Expr cond;
        auto conj = [&](Expr c) { cond = cond ? Expr(reffiner::_and(cond, c)) : c; };
        for (;;) {
            if (E->kind != NodeKind::SELECT) break;
            auto s = as<Select>(E);
            if (s->false_body.get() == ls.get()) {
                conj(s->cond);
                E = s->true_body;
            } else if (s->true_body.get() == ls.get()) {
                conj(reffiner::_not(s->cond));
                E = s->false_body;
            } else {
                throw LowerError("reduce accumulator field is not a conditional update of itself");
            }
        }
        if (E.get() == ls.get()) {
            lf.op = AggOp::NONE;
        } else if (E->kind == NodeKind::NARY) {
            auto n = as<NaryExpr>(E);
            auto a0 = n->args[0];
            auto a1 = n->args.size() > 1 ? n->args[1] : nullptr;
            switch (n->op) {
                case MathOp::ADD: {
                    // s + e, e + s, or a left-leaning chain s + e1 + e2 ...
                    std::vector<Expr> terms;
                    std::function<void(const Expr&)> chain = [&](const Expr& x) {
                        if (is_nary(x, MathOp::ADD)) {
                            chain(as<NaryExpr>(x)->args[0]);
                            terms.push_back(as<NaryExpr>(x)->args[1]);
                        } else {
                            terms.push_back(x);
                        }
                    };
                    if (a1 && a1.get() == ls.get()) {
                        lf.value = a0;
                    } else {
                        chain(E);
                        if (terms.empty() || terms[0].get() != ls.get())
                            throw LowerError("reduce sum is not of the form state + value");
                        Expr v = terms[1];
                        for (size_t i = 2; i < terms.size(); i++) v = reffiner::_add(v, terms[i]);
                        lf.value = v;
                    }
                    lf.op = AggOp::SUM;
                    break;
                }
                case MathOp::SUB:
                    if (a0.get() != ls.get()) throw LowerError("reduce difference is not state - value");
                    lf.value = reffiner::_neg(a1);
                    lf.op = AggOp::SUM;
                    break;
                case MathOp::MAX: case MathOp::MIN: case MathOp::OR: case MathOp::AND:
                    if (a0.get() == ls.get()) {
                        lf.value = a1;
                    } else if (a1.get() == ls.get()) {
                        lf.value = a0;
                        lf.state_first = false;
                    } else {
                        throw LowerError("reduce min/max/or/and does not take the state");
                    }
                    lf.op = n->op == MathOp::MAX ? AggOp::MAX : n->op == MathOp::MIN ? AggOp::MIN
                            : n->op == MathOp::OR ? AggOp::OR : AggOp::AND;
                    break;
                default: throw LowerError(std::string("reduce update operator not associative: ") + mathop_name(n->op));
            }
        } else {
            throw LowerError("reduce accumulator field is not an associative update");
        }
        lf.cond = cond;
        if (lf.op != AggOp::NONE) {
            if (mentions_state(lf.value) || (cond && mentions_state(cond)))
                throw LowerError("reduce update reads another state field");
            if (lf.op == AggOp::SUM && lf.value->kind == NodeKind::CONST && as<Const>(lf.value)->val == 1.0)
                lf.count = true;
            if (lf.op == AggOp::SUM && lf.type.btype == BOOL) throw LowerError("sum over bool");
        }
        if (mentions_state(lf.init)) throw LowerError("reduce init reads the state");
        out.push_back(lf);
    }

    // ---------------------------------------------------------------- grouping
    // Leaves whose conditions share the same filter conjuncts and differ only in
    // `key == constant` conjuncts over the same key expressions form dense groups.
    bool detect_groups(std::vector<Leaf>& leaves, std::vector<std::vector<int>>& groups,
                       std::vector<Expr>& key_exprs, std::vector<Expr>& filters)
    {
        std::vector<int> act;
        for (size_t i = 0; i < leaves.size(); i++)
            if (leaves[i].op != AggOp::NONE) act.push_back((int)i);
        if (act.size() < 2) return false;
        for (int i : act) {
            auto& lf = leaves[i];
            std::vector<Expr> cj;
            if (lf.cond) flatten_and(lf.cond, cj);
            for (auto& c : cj) {
                if (is_nary(c, MathOp::EQ)) {
                    auto n = as<NaryExpr>(c);
                    if (n->args[1]->kind == NodeKind::CONST && n->args[0]->kind != NodeKind::CONST) {
                        lf.keys.push_back({n->args[0], n->args[1]});
                        continue;
                    }
                    if (n->args[0]->kind == NodeKind::CONST && n->args[1]->kind != NodeKind::CONST) {
                        lf.keys.push_back({n->args[1], n->args[0]});
                        continue;
                    }
                }
                lf.filters.push_back(c);
            }
        }
        auto& l0 = leaves[act[0]];
        if (l0.keys.empty()) return false;
        // order keys by the first leaf's order; every leaf must have the same key expressions
        for (auto& kv : l0.keys) key_exprs.push_back(kv.first);
        for (int i : act) {
            auto& lf = leaves[i];
            if (lf.keys.size() != key_exprs.size() || lf.filters.size() != l0.filters.size()) return false;
            std::vector<std::pair<Expr, Expr>> ordered;
            for (auto& ke : key_exprs) {
                bool found = false;
                for (auto& kv : lf.keys)
                    if (same(kv.first, ke)) {
                        ordered.push_back(kv);
                        found = true;
                        break;
                    }
                if (!found) return false;
            }
            lf.keys = ordered;
            for (auto& f : lf.filters) {
                bool found = false;
                for (auto& g : l0.filters)
                    if (same(f, g)) found = true;
                if (!found) return false;
            }
        }
        filters = l0.filters;
        // partition by constant tuple, in first-appearance order
        std::vector<std::vector<double>> tuples;
        for (int i : act) {
            std::vector<double> t;
            for (auto& kv : leaves[i].keys) t.push_back(as<Const>(kv.second)->val);
            size_t g = 0;
            for (; g < tuples.size(); g++)
                if (tuples[g] == t) break;
            if (g == tuples.size()) {
                tuples.push_back(t);
                groups.emplace_back();
            }
            groups[g].push_back(i);
        }
        if (groups.size() < 2 || groups.size() > (size_t)RF_MAX_GROUPS_) return false;
        // every group must aggregate the same sequence of (op, type, value)
        auto& g0 = groups[0];
        for (auto& g : groups) {
            if (g.size() != g0.size()) return false;
            for (size_t m = 0; m < g.size(); m++) {
                auto &a = leaves[g[m]], &b = leaves[g0[m]];
                if (a.op != b.op || a.type != b.type || a.count != b.count || a.state_first != b.state_first ||
                    !same(a.value, b.value))
                    return false;
            }
        }
        return true;
    }
    static constexpr int RF_MAX_GROUPS_ = 64;

    // ---------------------------------------------------------------- code generation helpers
    static std::string acc_ctype(const Leaf& lf)
    {
        if (lf.count) return "long long";
        if (lf.type.btype == BOOL) return "long long";
        if (lf.type.is_float()) return lf.type.btype == FLOAT32 ? "float" : "double";
        if (lf.type.is_unsigned()) return "unsigned long long";
        return "long long";
    }

    // identity for sums; for idempotent ops every partial starts at the init value
    std::string acc_start(Emitter& E, const Leaf& lf)
    {
        if (lf.op == AggOp::SUM) return "0";
        return "(" + acc_ctype(lf) + ")(" + E.ev(lf.init).c + ")";
    }

    static std::string combine_expr(const Leaf& lf, const std::string& a, const std::string& b)
    {
        switch (lf.op) {
            case AggOp::SUM: return "(" + a + " + " + b + ")";
            case AggOp::MAX: return lf.state_first ? "((" + a + " < " + b + ") ? " + b + " : " + a + ")"
                                                   : "((" + b + " < " + a + ") ? " + a + " : " + b + ")";
            case AggOp::MIN: return lf.state_first ? "((" + b + " < " + a + ") ? " + b + " : " + a + ")"
                                                   : "((" + a + " < " + b + ") ? " + a + " : " + b + ")";
            case AggOp::OR: return "(long long)((" + a + ") || (" + b + "))";
            case AggOp::AND: return "(long long)((" + a + ") && (" + b + "))";
            default: return a;
        }
    }

    // final state value of a leaf from its folded accumulator `tot`
    std::string final_leaf(Emitter& E, const Leaf& lf, const std::string& tot)
    {
        std::string T = ctype(lf.type);
        if (lf.op == AggOp::NONE) return "((" + T + ")(" + E.ev(lf.init).c + "))";
        if (lf.op == AggOp::SUM) return "((" + T + ")((" + E.ev(lf.init).c + ") + (" + T + ")(" + tot + ")))";
        return "((" + T + ")(" + tot + "))";
    }

    // evaluates the Func output with the Reduce bound to its final state; stores in C layout
    void emit_output_store(Emitter& E, std::ostringstream& o, const Reduce& red,
                           const std::map<std::vector<size_t>, std::string>& finals)
    {
        std::function<Val(const DataType&, std::vector<size_t>)> mk = [&](const DataType& t, std::vector<size_t> p) {
            if (t.is_struct()) {
                Val v;
                v.k = Val::STRUCT;
                v.type = t;
                for (size_t i = 0; i < t.dtypes.size(); i++) {
                    auto q = p;
                    q.push_back(i);
                    v.f.push_back(mk(t.dtypes[i], q));
                }
                return v;
            }
            Val v;
            v.c = finals.at(p);
            v.type = t;
            return v;
        };
        Val st = mk(red.type, {});
        // bind every symbol whose table entry is this Reduce
        for (auto& kv : fn_->tbl)
            if (resolve(kv.first).get() == (const ExprNode*)&red) E.bind(kv.first, st);
        Expr outx = fn_->output;
        Val ov;
        if ((const ExprNode*)resolve(outx).get() == (const ExprNode*)&red) ov = st;
        else ov = E.ev(outx);
        for (auto& d : E.decls) o << "    " << d << "\n";
        E.decls.clear();
        size_t off = 0;
        store_c(o, ov, plan_.out_type, off, "out");
        plan_.out_size = c_size(plan_.out_type);
    }

    void store_c(std::ostringstream& o, const Val& v, const DataType& t, size_t& off, const std::string& base)
    {
        if (t.is_struct()) {
            size_t al = c_align(t);
            off = (off + al - 1) / al * al;
            size_t start = off;
            for (size_t i = 0; i < t.dtypes.size(); i++) store_c(o, v.f.at(i), t.dtypes[i], off, base);
            off = start + c_size(t);
            return;
        }
        size_t al = c_align(t);
        off = (off + al - 1) / al * al;
        o << "    *(" << ctype(t) << "*)(" << base << " + " << off << ") = (" << ctype(t) << ")(" << v.c << ");\n";
        off += c_size(t);
    }

    // ---------------------------------------------------------------- driving loop of a Reduce
    struct Drive {
        bool subvec = false;
        Space sp;
        int input = -1;
        int slot = -1;
    };

    // binds the reduce value symbol and emits the row prologue (validity / iteration condition);
    // returns the row-condition expression
    std::string bind_row(Emitter& E, const Reduce& red, const Drive& d, std::ostringstream& body)
    {
        bind_inputs(E);
        std::string sl = std::to_string(d.slot);
        if (d.subvec) {
            // LoopGen::visit(Reduce) over a SubVector: value = columns 1..n-1, condition = validity
            // of column 1 (loopgen.cpp:221-242)
            const DataType& vt = fn_->inputs[d.input]->type;
            Val v;
            v.k = Val::STRUCT;
            v.type = red.val->type;
            for (size_t c = 1; c < vt.dtypes.size(); c++) {
                v.f.push_back(E.scalar("rf_ld<" + ctype(vt.dtypes[c]) + ">(P.t[" + sl + "].col[" + std::to_string(c) +
                                           "].data, r)",
                                       vt.dtypes[c]));
            }
            E.bind(red.val, v);
            pending_cols_ = true;
            return "rf_valid(P.t[" + sl + "].col[1].valid, r)";
        }
        // Op iteration space (single iterator)
        const auto& op = *as<Op>(red.vec);
        const Space& sp = d.sp;
        std::string it_c, cond;
        std::string T = ctype(sp.iter->type);
        if (sp.has_vec) {
            note_col(d.input, 0);
            it_c = "rf_ld<" + T + ">(P.t[" + sl + "].col[0].data, r)";
            cond = "rf_valid(P.t[" + sl + "].col[0].valid, r)";
            E.vec_iter_idx[{sp.vec_node.get(), sp.iter.get()}] = "r";
        } else {
            it_c = "((" + T + ")r)";
            cond = "true";
        }
        body << "    const " << T << " it = " << it_c << ";\n";
        E.bind(op.iters[0], E.scalar("it", sp.iter->type));
        if (!sp.lbs.empty()) cond += " && (it >= (" + T + ")P.range[2])";
        if (!sp.ubs.empty()) cond += " && (it <= (" + T + ")P.range[3])";
        for (auto& f : sp.filters) cond += " && (" + E.ev(f).c + ")";
        // value = (iterators..., outputs...)  (loopgen.cpp:88-91)
        Val v;
        v.k = Val::STRUCT;
        v.type = red.val->type;
        v.f.push_back(E.scalar("it", sp.iter->type));
        for (auto& o : op.outputs) v.f.push_back(E.ev(o));
        E.bind(red.val, v);
        return cond;
    }
    bool pending_cols_ = false;

    // range kernels of an Op iteration space: start = Locate(max(lbs, col0[0])) for a vector,
    // end = first row past the upper bound (UBoundSpace::_is_alive stops the loop there)
    void emit_range_kernels(std::ostringstream& o, const Drive& d)
    {
        const Space& sp = d.sp;
        Emitter E(*this);
        bind_inputs(E);
        std::string T = ctype(sp.iter->type);
        std::string sl = std::to_string(d.slot);
        std::ostringstream b;
        if (sp.has_vec) {
            std::string first = "rf_rd<" + T + ">(P.t[" + sl + "].col[0], 0)";
            std::string last = "rf_rd<" + T + ">(P.t[" + sl + "].col[0], P.t[" + sl + "].col[0].len - 1)";
            std::string L = bound_expr(E, sp.lbs, first, true, sp.iter->type);
            std::string U = sp.ubs.empty() ? "0" : bound_expr(E, sp.ubs, last, false, sp.iter->type);
            plan_.needs_index[d.input] = 1;
            b << "    const " << T << " L = " << L << ";\n";
            b << "    const " << T << " U = " << U << ";\n";
            b << "    long long start = P.t[" << sl << "].col[0].len > 0 ? rf_locate(P.t[" << sl << "].ix, (long long)L) : 0;\n";
            b << "    long long end = P.t[" << sl << "].col[0].len;\n";
            b << "    if (start < 0) { rf_set_err(P, RF_DEVERR_RANGE); start = end; }\n";
        } else {
            std::string L = bound_expr(E, sp.lbs, "", true, sp.iter->type);
            std::string U = bound_expr(E, sp.ubs, "", false, sp.iter->type);
            b << "    const " << T << " L = " << L << ";\n";
            b << "    const " << T << " U = " << U << ";\n";
            b << "    long long start = (long long)L;\n";
            b << "    long long end = (long long)U + 1;\n";
            b << "    if (end < start) end = start;\n";
        }
        o << "extern \"C\" __global__ void rf_range(const __grid_constant__ RfParams P)\n{\n";
        o << "    if (threadIdx.x != 0 || blockIdx.x != 0) return;\n";
        for (auto& dcl : E.decls) o << "    " << dcl << "\n";
        o << b.str();
        o << "    P.range[0] = start;\n    P.range[1] = end;\n    P.range[2] = (long long)L;\n    P.range[3] = (long long)U;\n}\n\n";
        plan_.kernels.push_back({"rf_range", 32, 0, KernelSpec::RANGE});
        if (sp.has_vec && !sp.ubs.empty()) {
            o << "extern \"C\" __global__ void __launch_bounds__(256) rf_stop(const __grid_constant__ RfParams P)\n{\n";
            o << "    const long long start = P.range[0], n = P.t[" << sl << "].col[0].len;\n";
            o << "    const " << T << " U = (" << T << ")P.range[3];\n";
            o << "    for (long long r = start + blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n;\n"
              << "         r += (long long)gridDim.x * blockDim.x) {\n";
            o << "        if (!(rf_ld<" << T << ">(P.t[" << sl << "].col[0].data, r) <= U)) { atomicMin(P.range + 1, r); break; }\n";
            o << "    }\n}\n\n";
            plan_.kernels.push_back({"rf_stop", 256, 0, KernelSpec::STOP});
        }
        plan_.device_range = true;
    }

    // ---------------------------------------------------------------- Reduce lowering
    void lower_reduce(const Reduce& red)
    {
        Drive d;
        if (red.vec->kind == NodeKind::OP) {
            d.sp = op_space(*as<Op>(red.vec));
            if (d.sp.n_vecs > 1) throw LowerError("a Reduce over a merge co-iteration is not lowered");
            if (d.sp.has_vec) {
                d.input = d.sp.vec_input;
                d.slot = plan_.table_slot[d.input];
                plan_.drive_input = d.input;
                HostExpr lo;
                lo.kind = HostExpr::CONST;
                lo.value = 0;
                HostExpr hi;
                hi.kind = HostExpr::LEN;
                hi.input = d.input;
                hi.col = 0;
                plan_.row_lo = lo;
                plan_.row_hi = hi;
            } else {
                // range space: bounds are host-evaluable; the device range kernel still computes
                // them (exactly as the loop would) and the host passes a safe tiling range
                plan_.row_lo = minmax_host(d.sp.lbs, true);
                HostExpr hi = minmax_host(d.sp.ubs, false);
                HostExpr one;
                one.kind = HostExpr::CONST;
                one.value = 1;
                HostExpr h2;
                h2.kind = HostExpr::ADD;
                h2.args = {hi, one};
                plan_.row_hi = h2;
            }
        } else if (red.vec->kind == NodeKind::SUBVECTOR) {
            auto sv = as<SubVector>(red.vec);
            auto f = input_index_.find(resolve(sv->vec).get());
            if (f == input_index_.end()) throw LowerError("reduce over a subvector of a non-input vector");
            d.subvec = true;
            d.input = f->second;
            d.slot = plan_.table_slot[d.input];
            plan_.drive_input = d.input;
            plan_.row_lo = host_expr(sv->start);
            plan_.row_hi = host_expr(sv->end);
            note_col(d.input, 1);
        } else {
            throw LowerError("Unsupported reduction vector");  // loopgen.cpp:243-245
        }

        std::vector<Leaf> leaves;
        collect_leaves(red, red.type, {}, leaves);
        std::vector<std::vector<int>> groups;
        std::vector<Expr> key_exprs, filters;
        bool grouped = detect_groups(leaves, groups, key_exprs, filters);

        std::ostringstream src;
        src << "// generated by the reffine_gb300 lowering pass: " << fn_->name << "\n";
        src << "#include \"rf_device.cuh\"\n\n";
        if (!d.subvec) emit_range_kernels(src, d);

        if (!grouped) gen_scan_reduce(src, red, d, leaves);
        else gen_group_reduce(src, red, d, leaves, groups, key_exprs, filters);
        plan_.source = src.str();
    }

    HostExpr minmax_host(const std::vector<Expr>& bs, bool is_max)
    {
        HostExpr r = host_expr(bs[0]);
        for (size_t i = 1; i < bs.size(); i++) {
            HostExpr h;
            h.kind = is_max ? HostExpr::MAX : HostExpr::MIN;
            h.args = {host_expr(bs[i]), r};
            r = h;
        }
        return r;
    }

    // Loads of the driving row (rf_ld<T>(P.t[s].col[c].data, r)) that a condition reads are
    // issued together at the top of the row function instead of one after another inside the
    // short-circuit chain; `code` pieces are rewritten to use the hoisted locals.
    static std::string hoist_row_loads(const std::string& cond, std::vector<std::string*> code)
    {
        std::ostringstream decl;
        std::map<std::string, std::string> seen;
        const std::string pat = "rf_ld<";
        for (size_t pos = cond.find(pat); pos != std::string::npos; pos = cond.find(pat, pos + 1)) {
            size_t e = cond.find(", r)", pos);
            if (e == std::string::npos) continue;
            std::string call = cond.substr(pos, e + 4 - pos);
            if (call.find("P.t[") == std::string::npos || call.find('(', pat.size()) == std::string::npos) continue;
            if (seen.count(call)) continue;
            std::string ty = call.substr(pat.size(), call.find('>') - pat.size());
            std::string nm = "ld" + std::to_string(seen.size());
            seen[call] = nm;
            decl << "    const " << ty << " " << nm << " = " << call << ";\n";
        }
        for (auto* c : code)
            for (auto& kv : seen) {
                size_t p;
                while ((p = c->find(kv.first)) != std::string::npos) c->replace(p, kv.first.size(), kv.second);
            }
        return decl.str();
    }

    // Loads of the driving row that a row's values read once it has passed its filter (text
    // from position `from` on): each distinct load into one local, declared at `from`, so the
    // compiler sees equal operands and computes a shared subexpression (price * (1 - disc) in
    // two sums) once.  Same loads, same rounding: only repeated work goes.
    static void hoist_value_loads(std::string& text, size_t from)
    {
        const std::string pat = "rf_ld<";
        std::map<std::string, std::string> seen;
        std::vector<std::string> order;
        for (size_t pos = text.find(pat, from); pos != std::string::npos; pos = text.find(pat, pos + 1)) {
            size_t e = text.find(", r)", pos);
            if (e == std::string::npos) continue;
            std::string call = text.substr(pos, e + 4 - pos);
            if (call.find("P.t[") == std::string::npos || call.find('(', pat.size()) == std::string::npos) continue;
            if (seen.count(call)) continue;
            seen[call] = "lv" + std::to_string(order.size());
            order.push_back(call);
        }
        if (order.empty()) return;
        std::ostringstream decl;
        for (auto& c : order) decl << "    const " << c.substr(pat.size(), c.find('>') - pat.size()) << " " << seen[c] << " = " << c << ";\n";
        std::string tail = text.substr(from);
        for (auto& c : order) {
            size_t p;
            while ((p = tail.find(c)) != std::string::npos) tail.replace(p, c.size(), seen[c]);
        }
        text = text.substr(0, from) + decl.str() + tail;
    }

    // cost-ordered conjunction: cheap column predicates first, hash probes last
    // evaluation cost class of a condition: 1 per node, 20 per element or data read, 100 per
    // index probe (Locate)
    int cost_of(const Expr& x)
    {
        std::set<const ExprNode*> seen;
        return cost_rec(x, seen);
    }

    int cost_rec(const Expr& e, std::set<const ExprNode*>& seen)
    {
        if (!e || seen.count(e.get())) return 0;
        seen.insert(e.get());
        int k = e->kind == NodeKind::LOCATE ? 100 : e->kind == NodeKind::READDATA ? 20 : 1;
        if (e->kind == NodeKind::SYM) {
            auto it = fn_->tbl.find(std::static_pointer_cast<SymNode>(e));
            if (it != fn_->tbl.end()) return cost_rec(it->second, seen);
            return 0;
        }
        if (e->kind == NodeKind::ELEMENT) k = 20;
        std::vector<Expr> ch;
        children(e, ch);
        for (auto& x : ch) k += cost_rec(x, seen);
        return k;
    }

    Expr order_conjuncts(const Expr& c)
    {
        std::vector<Expr> cj;
        flatten_and(c, cj);
        if (cj.size() < 2) return c;
        std::function<int(const Expr&, std::set<const ExprNode*>&)> cost = [&](const Expr& e, std::set<const ExprNode*>& seen) -> int {
            if (!e || seen.count(e.get())) return 0;
            seen.insert(e.get());
            int k = e->kind == NodeKind::LOCATE ? 100 : e->kind == NodeKind::READDATA ? 20 : 1;
            if (e->kind == NodeKind::SYM) {
                auto it = fn_->tbl.find(std::static_pointer_cast<SymNode>(e));
                if (it != fn_->tbl.end()) return cost(it->second, seen);
                return 0;
            }
            if (e->kind == NodeKind::ELEMENT) k = 20;
            std::vector<Expr> ch;
            children(e, ch);
            for (auto& x : ch) k += cost(x, seen);
            return k;
        };
        std::vector<std::pair<int, Expr>> v;
        for (auto& x : cj) {
            std::set<const ExprNode*> seen;
            v.push_back({cost(x, seen), x});
        }
        std::stable_sort(v.begin(), v.end(), [](auto& a, auto& b) { return a.first < b.first; });
        Expr r = v[0].second;
        for (size_t i = 1; i < v.size(); i++) r = reffiner::_and(r, v[i].second);
        return r;
    }

    // RfAcc (one 8-byte slot per active leaf), rf_acc_init, rf_acc_combine, rf_acc_shfl
    void emit_acc(std::ostringstream& src, std::vector<Leaf>& leaves, const std::vector<int>& act)
    {
        std::ostringstream acc, init, comb, shfl;
        Emitter Ei(*this);
        bind_inputs(Ei);
        acc << "struct RfAcc {\n";
        if (act.empty()) acc << "    long long unused;\n";
        for (size_t k = 0; k < act.size(); k++) {
            auto& lf = leaves[act[k]];
            std::string ct = acc_ctype(lf);
            if (ct == "float") ct = "double";  // keep 8-byte slots; f32 sums are rounded per update below
            acc << "    " << ct << " a" << k << ";\n";
        }
        acc << "};\n\n";
        init << "RF_DEV void rf_acc_init(const RfParams& P, RfAcc& A)\n{\n";
        std::ostringstream initb;
        for (size_t k = 0; k < act.size(); k++) initb << "    A.a" << k << " = " << acc_start(Ei, leaves[act[k]]) << ";\n";
        for (auto& dcl : Ei.decls) init << "    " << dcl << "\n";
        init << initb.str() << "}\n\n";
        comb << "RF_DEV void rf_acc_combine(RfAcc& A, const RfAcc& B)\n{\n";
        for (size_t k = 0; k < act.size(); k++) {
            auto& lf = leaves[act[k]];
            std::string a = "A.a" + std::to_string(k), b = "B.a" + std::to_string(k);
            std::string e = combine_expr(lf, a, b);
            if (lf.type.btype == FLOAT32 && lf.op == AggOp::SUM) e = "(double)((float)" + a + " + (float)" + b + ")";
            comb << "    " << a << " = " << e << ";\n";
        }
        if (act.empty()) comb << "    (void)A; (void)B;\n";
        comb << "}\n\n";
        shfl << "RF_DEV RfAcc rf_acc_shfl(const RfAcc& A, int off)\n{\n    RfAcc R;\n";
        for (size_t k = 0; k < act.size(); k++) shfl << "    R.a" << k << " = __shfl_down_sync(0xffffffffu, A.a" << k << ", off);\n";
        if (act.empty()) shfl << "    R.unused = A.unused; (void)off;\n";
        shfl << "    return R;\n}\n\n";
        src << acc.str() << init.str() << comb.str() << shfl.str();
    }

    // rf_row: one row of the driving loop folded into the accumulator
    void emit_row(std::ostringstream& src, const Reduce& red, const Drive& d, std::vector<Leaf>& leaves,
                  const std::vector<int>& act)
    {
        std::ostringstream row;
        Emitter E(*this);
        std::ostringstream body;
        std::string rowcond = bind_row(E, red, d, body);
        // leaves sharing a condition (structurally) are updated under one test of it
        std::ostringstream upd;
        std::string allconds;
        std::vector<char> done(act.size(), 0);
        for (size_t k = 0; k < act.size(); k++) {
            if (done[k]) continue;
            auto& lf = leaves[act[k]];
            std::string cond = lf.cond ? E.ev(order_conjuncts(lf.cond)).c : "";
            allconds += cond;
            std::string ind = cond.empty() ? "    " : "        ";
            if (!cond.empty()) upd << "    if (" << cond << ") {\n";
            for (size_t j = k; j < act.size(); j++) {
                auto& lj = leaves[act[j]];
                if (done[j]) continue;
                bool samec = (!lf.cond && !lj.cond) || (lf.cond && lj.cond && same(lf.cond, lj.cond));
                if (!samec) continue;
                done[j] = 1;
                std::string a = "A.a" + std::to_string(j);
                std::string val;
                if (lj.count) val = "1";
                else if (lj.op == AggOp::OR || lj.op == AggOp::AND) val = "(long long)(" + E.ev(lj.value).c + ")";
                else val = "(" + ctype(lj.type) + ")(" + E.ev(lj.value).c + ")";
                std::string e = combine_expr(lj, a, val);
                if (lj.type.btype == FLOAT32 && lj.op == AggOp::SUM) e = "(double)((float)" + a + " + " + val + ")";
                upd << ind << a << " = " << e << ";\n";
            }
            if (!cond.empty()) upd << "    }\n";
        }
        std::string updates = upd.str();
        std::vector<std::string> dcls(E.decls.begin(), E.decls.end());
        std::vector<std::string*> pieces{&rowcond, &updates};
        for (auto& d : dcls) pieces.push_back(&d);
        // a scan's row reads every column it references up front, the columns its values read
        // too (not after the filter passes: a load issued only then is a second round trip to
        // memory per row, and the 4-row vector loads fetch whole sectors anyway)
        std::string condtext = rowcond + allconds + updates;
        std::string hoisted = hoist_row_loads(condtext, pieces);
        // the hoisted loads ("    const T ldK = rf_ld<T>(COL.data, r);") become parameters of the
        // row body rf_row_v, so that rf_row (one row) and rf_row4 (4 rows from vector loads) share it
        std::vector<std::array<std::string, 3>> hl;  // type, name, column pointer
        {
            std::istringstream in(hoisted);
            std::string line;
            while (std::getline(in, line)) {
                size_t c = line.find("const "), eq = line.find(" = rf_ld<"), open = line.find(">(", eq);
                size_t end = line.rfind(", r);");
                if (c == std::string::npos || eq == std::string::npos || open == std::string::npos || end == std::string::npos) {
                    hl.clear();
                    break;
                }
                std::string decl = line.substr(c + 6, eq - c - 6);
                size_t sp = decl.rfind(' ');
                hl.push_back({decl.substr(0, sp), decl.substr(sp + 1), line.substr(open + 2, end - open - 2)});
            }
        }
        const bool vec4 = !hl.empty() && plan_.kind == PlanKind::SCAN_REDUCE;
        if (vec4) {
            row << "RF_DEV void rf_row_v(const RfParams& P, long long r, RfAcc& A";
            for (auto& h : hl) row << ", const " << h[0] << " " << h[1];
            row << ")\n{\n" << body.str();
        } else {
            row << "RF_DEV void rf_row(const RfParams& P, long long r, RfAcc& A)\n{\n";
            row << body.str() << hoisted;
        }
        for (auto& dcl : dcls) row << "    " << dcl << "\n";
        row << "    if (!(" << rowcond << ")) return;\n";
        row << updates;
        if (act.empty()) row << "    (void)A;\n";
        row << "}\n\n";
        if (vec4) {
            row << "RF_DEV void rf_row(const RfParams& P, long long r, RfAcc& A)\n{\n" << hoisted;
            row << "    rf_row_v(P, r, A";
            for (auto& h : hl) row << ", " << h[1];
            row << ");\n}\n\n";
            row << "#define RF_VEC4 1\n";
            row << "RF_DEV void rf_row4(const RfParams& P, long long r, RfAcc& A)\n{\n";
            for (auto& h : hl) {
                // bool columns are read as bytes (any nonzero byte is true, as rf_ld<bool> reads them)
                std::string lt = h[0] == "bool" ? "int8_t" : h[0];
                row << "    " << lt << " " << h[1] << "[4];\n    rf_ld4<" << lt << ">(" << h[2] << ", r, " << h[1] << ");\n";
            }
            for (int q = 0; q < 4; q++) {
                row << "    rf_row_v(P, r + " << q << ", A";
                for (auto& h : hl) row << ", " << (h[0] == "bool" ? "(" + h[1] + "[" + std::to_string(q) + "] != 0)"
                                                              : h[1] + "[" + std::to_string(q) + "]");
                row << ");\n";
            }
            row << "}\n\n";
        }
        src << row.str();
    }

    void gen_scan_reduce(std::ostringstream& src, const Reduce& red, const Drive& d, std::vector<Leaf>& leaves)
    {
        plan_.kind = PlanKind::SCAN_REDUCE;
        const int T = plan_.threads;
        std::vector<int> act;
        for (size_t i = 0; i < leaves.size(); i++)
            if (leaves[i].op != AggOp::NONE) act.push_back((int)i);
        emit_acc(src, leaves, act);
        emit_row(src, red, d, leaves, act);
        std::ostringstream fin;

        // epilogue
        Emitter Ef(*this);
        bind_inputs(Ef);
        std::map<std::vector<size_t>, std::string> finals;
        std::ostringstream fb;
        for (size_t i = 0, k = 0; i < leaves.size(); i++) {
            auto& lf = leaves[i];
            std::string tot = lf.op == AggOp::NONE ? "0" : "A.a" + std::to_string(k++);
            std::string nm = "st" + std::to_string(i);
            fb << "    const " << ctype(lf.type) << " " << nm << " = " << final_leaf(Ef, lf, tot) << ";\n";
            finals[lf.path] = nm;
        }
        fin << "RF_DEV void rf_finish(const RfParams& P, const RfAcc& A, unsigned char* out)\n{\n";
        std::ostringstream stores;
        emit_output_store(Ef, stores, red, finals);
        for (auto& dcl : Ef.decls) fin << "    " << dcl << "\n";
        fin << fb.str() << stores.str() << "}\n\n";

        src << fin.str();
        src << "#define RF_SCAN_REDUCE 1\n#include \"rf_templates.cuh\"\n";
        src << "RF_SCAN_REDUCE_KERNEL(rf_main, " << T << ")\n";
        plan_.kernels.push_back({"rf_main", T, 0, KernelSpec::MAIN});
        plan_.acc_bytes = std::max<size_t>(8, act.size() * 8);
    }

    // --------------------------------------------------------------- index filter pushdown
    // A filter conjunct that depends only on the row an index probe found - data of the probed
    // table read at the Locate, constants, scalar inputs - can be evaluated when the index is
    // built: a run builds a smaller index holding only the entries whose row passes, so the
    // probes touch a table that may fit in L2.  The conjunct stays in the row filter, so a run
    // on the full index (a batched run, rf_plan_run_noalloc) gives the same result.
    bool ixf_analyze(const Expr& e, std::vector<Expr>& locs, std::set<const ExprNode*>& seen)
    {
        if (!e || seen.count(e.get())) return true;
        seen.insert(e.get());
        switch (e->kind) {
            case NodeKind::CONST: return true;
            case NodeKind::LOCATE: locs.push_back(e); return true;
            case NodeKind::READDATA: {
                Expr idx = as<ReadData>(e)->idx;
                while (idx->kind == NodeKind::SYM) {
                    auto it = fn_->tbl.find(std::static_pointer_cast<SymNode>(idx));
                    if (it == fn_->tbl.end()) return false;
                    idx = it->second;
                }
                if (idx->kind != NodeKind::LOCATE) return false;
                if (!same(as<ReadData>(e)->vec, as<Locate>(idx)->vec)) return false;
                locs.push_back(idx);
                return true;
            }
            case NodeKind::SYM: {
                auto it = fn_->tbl.find(std::static_pointer_cast<SymNode>(e));
                if (it != fn_->tbl.end()) return ixf_analyze(it->second, locs, seen);
                for (auto& in : fn_->inputs)
                    if (in.get() == e.get()) return e->type.is_primitive();  // a scalar argument
                return false;
            }
            case NodeKind::NARY: case NodeKind::SELECT: case NodeKind::CAST: {
                std::vector<Expr> ch;
                children(e, ch);
                for (auto& c : ch)
                    if (!ixf_analyze(c, locs, seen)) return false;
                return true;
            }
            default: return false;
        }
    }

    void all_locates(const Expr& e, std::vector<Expr>& out, std::set<const ExprNode*>& seen)
    {
        if (!e || seen.count(e.get())) return;
        seen.insert(e.get());
        if (e->kind == NodeKind::LOCATE) out.push_back(e);
        if (e->kind == NodeKind::SYM) {
            auto it = fn_->tbl.find(std::static_pointer_cast<SymNode>(e));
            if (it != fn_->tbl.end()) all_locates(it->second, out, seen);
            return;
        }
        std::vector<Expr> ch;
        children(e, ch);
        for (auto& c : ch) all_locates(c, out, seen);
    }

    void push_index_filter(std::ostringstream& o, const Reduce& red, const std::vector<Expr>& filters)
    {
        if (filters.empty()) return;
        Expr f = filters[0];
        for (size_t i = 1; i < filters.size(); i++) f = reffiner::_and(f, filters[i]);
        std::vector<Expr> cj;
        flatten_and(f, cj);
        Expr L;
        std::vector<Expr> pushed, locs;
        for (auto& c : cj) {
            std::vector<Expr> l;
            std::set<const ExprNode*> seen;
            if (!ixf_analyze(c, l, seen) || l.empty()) continue;
            bool one = true;
            for (auto& x : l) one = one && same(x, L ? L : l[0]);
            if (!one) continue;
            if (!L) L = l[0];
            pushed.push_back(c);
            locs.insert(locs.end(), l.begin(), l.end());
        }
        if (!L) return;
        // the probed table must be an input with no other probe into it in the plan
        Expr vec = as<Locate>(L)->vec;
        int input = -1;
        for (size_t i = 0; i < fn_->inputs.size(); i++)
            if (fn_->inputs[i].get() == vec.get()) input = (int)i;
        if (input < 0) return;
        std::vector<Expr> every;
        std::set<const ExprNode*> seen;
        all_locates(red.acc_expr, every, seen);
        for (auto& x : filters) all_locates(x, every, seen);
        for (auto& x : every)
            if (same(as<Locate>(x)->vec, vec) && !same(x, L)) return;
        Emitter Ek(*this);
        bind_inputs(Ek);
        for (auto& x : locs) Ek.node_bind[x.get()] = Ek.scalar("row", types::IDX_T);
        Expr pf = pushed[0];
        for (size_t i = 1; i < pushed.size(); i++) pf = reffiner::_and(pf, pushed[i]);
        std::string kc = Ek.ev(pf).c;
        const std::string S = std::to_string(plan_.table_slot[input]);
        o << "// the probed table's index entries whose row passes the pushed-down filter\n";
        o << "RF_DEV bool rf_ixf_keep(const RfParams& P, long long row)\n{\n";
        for (auto& dcl : Ek.decls) o << "    " << dcl << "\n";
        o << "    return " << kc << ";\n}\n\n";
        o << "#define RF_IXF_SLOT " << S << "\n";
        o << R"(// Entries to index, 4 per thread per step.  aux_n1 == 0: the slots of the table's full index
// (each key with the row the full index returns for it); aux_n1 == 1: the table's rows (when no
// key repeats, the same entries, from the smaller table).  The empty key's row comes from the
// full index's special slot in the first mode and from its row in the second.
RF_DEV bool rf_ixf_entry(const RfParams& P, unsigned long long i, long long& key, long long& row)
{
    const RfIndex& ix = P.t[RF_IXF_SLOT].ix;
    if (P.aux_n1 == 0) {
        if (i >= ix.cap) return false;
        const longlong2 v = __ldg((const longlong2*)ix.slots + i);
        key = v.x;
        row = v.y;
        return v.x != RF_EMPTY_KEY;
    }
    const RfCol& c = P.t[RF_IXF_SLOT].col[0];
    if ((long long)i >= c.len || !rf_valid(c.valid, (long long)i)) return false;
    key = __ldcs((const long long*)c.data + i);
    row = (long long)i;
    return key != RF_EMPTY_KEY;
}

RF_DEV unsigned long long rf_ixf_n(const RfParams& P)
{
    return P.aux_n1 == 0 ? P.t[RF_IXF_SLOT].ix.cap : (unsigned long long)P.t[RF_IXF_SLOT].col[0].len;
}

// the empty key's row (the full index keeps its first row in both modes)
RF_DEV long long rf_ixf_special(const RfParams& P) { return *P.t[RF_IXF_SLOT].ix.special; }

// count of the entries to keep (aux2)
extern "C" __global__ void __launch_bounds__(256) rf_ixf_count(const __grid_constant__ RfParams P)
{
    const unsigned long long n = rf_ixf_n(P), stride = gridDim.x * 256ull * 4;
    unsigned long long c = 0;
    for (unsigned long long b = blockIdx.x * 256ull * 4 + threadIdx.x; b < n; b += stride) {
        long long k[4], r[4];
        bool ok[4];
#pragma unroll
        for (int j = 0; j < 4; j++) ok[j] = rf_ixf_entry(P, b + j * 256ull, k[j], r[j]);
#pragma unroll
        for (int j = 0; j < 4; j++) c += ok[j] && rf_ixf_keep(P, r[j]);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const long long r = rf_ixf_special(P);
        if (r != RF_INT64_MAX && rf_ixf_keep(P, r)) c++;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) c += __shfl_down_sync(0xffffffffu, c, off);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd((unsigned long long*)P.aux2, c);
}

// the filtered index: aux_n0 slots at aux0, its empty-key row at aux1
extern "C" __global__ void __launch_bounds__(256) rf_ixf_init(const __grid_constant__ RfParams P)
{
    longlong2* t = (longlong2*)P.aux0;
    for (long long i = blockIdx.x * 256ll + threadIdx.x; i < P.aux_n0; i += gridDim.x * 256ll) t[i] = make_longlong2(RF_EMPTY_KEY, 0);
    if (blockIdx.x == 0 && threadIdx.x == 0) *(long long*)P.aux1 = RF_INT64_MAX;
}

extern "C" __global__ void __launch_bounds__(256) rf_ixf_build(const __grid_constant__ RfParams P)
{
    longlong2* t = (longlong2*)P.aux0;
    const unsigned long long C = (unsigned long long)P.aux_n0;
    const unsigned long long n = rf_ixf_n(P), stride = gridDim.x * 256ull * 4;
    for (unsigned long long b = blockIdx.x * 256ull * 4 + threadIdx.x; b < n; b += stride) {
        long long k[4], r[4];
        bool ok[4];
#pragma unroll
        for (int j = 0; j < 4; j++) ok[j] = rf_ixf_entry(P, b + j * 256ull, k[j], r[j]);
        // the four entries probe in rounds: each round issues their compare-and-swaps together
        // (independent atomics in flight), then moves the ones that met a taken slot on by one
        unsigned long long h[4];
        bool pend[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            pend[j] = ok[j] && rf_ixf_keep(P, r[j]);
            h[j] = pend[j] ? rf_home(k[j], C) : 0;
        }
        for (unsigned long long m = 0; m < C && (pend[0] || pend[1] || pend[2] || pend[3]); ++m) {
            unsigned long long prev[4];
#pragma unroll
            for (int j = 0; j < 4; j++)
                prev[j] = pend[j] ? atomicCAS((unsigned long long*)&t[h[j]].x, (unsigned long long)RF_EMPTY_KEY,
                                              (unsigned long long)k[j])
                                  : 0ULL;
#pragma unroll
            for (int j = 0; j < 4; j++) {
                if (!pend[j]) continue;
                if (prev[j] == (unsigned long long)RF_EMPTY_KEY) {
                    t[h[j]].y = r[j];
                    pend[j] = false;
                } else if (++h[j] == C) {
                    h[j] = 0;
                }
            }
        }
        if (pend[0] || pend[1] || pend[2] || pend[3]) rf_set_err(P, RF_DEVERR_OVERFLOW);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const long long r = rf_ixf_special(P);
        if (r != RF_INT64_MAX && rf_ixf_keep(P, r)) *(long long*)P.aux1 = r;
    }
}

)";
        plan_.ixf_input = input;
        plan_.kernels.push_back({"rf_ixf_count", 256, 0, KernelSpec::IXCOUNT});
        plan_.kernels.push_back({"rf_ixf_init", 256, 0, KernelSpec::IXINIT});
        plan_.kernels.push_back({"rf_ixf_build", 256, 0, KernelSpec::IXBUILD});
    }

    // RF_PREFETCH: rf_prefetch_rows(P, r0, r1) bulk-prefetches into L2 the rows [r0, r1) of every
    // column `row` (a row function's text) reads at the loop's own row r, i.e. every
    // rf_ld<T>(P.t[slot].col[c].data, r).  Returns false when there is none.
    bool emit_prefetch(std::ostringstream& src, const std::string& row, int slot)
    {
        static const std::map<std::string, int> sizes = {
            {"bool", 1}, {"int8_t", 1}, {"uint8_t", 1}, {"int16_t", 2}, {"uint16_t", 2}, {"int32_t", 4},
            {"uint32_t", 4}, {"float", 4}, {"int64_t", 8}, {"uint64_t", 8}, {"double", 8}};
        const std::string pre = "rf_ld<", mid = "(P.t[" + std::to_string(slot) + "].col[";
        std::vector<std::pair<std::string, int>> cols;
        for (size_t at = row.find(pre); at != std::string::npos; at = row.find(pre, at + pre.size())) {
            size_t te = row.find('>', at);
            if (te == std::string::npos) break;
            auto sz = sizes.find(row.substr(at + pre.size(), te - at - pre.size()));
            size_t ce = row.find(", r)", te);
            if (sz == sizes.end() || ce == std::string::npos) continue;
            std::string arg = row.substr(te + 1, ce - te - 1);
            if (arg.size() <= mid.size() + 5 || arg.compare(0, mid.size(), mid) != 0 ||
                arg.compare(arg.size() - 5, 5, ".data") != 0 || arg.find_first_of(" ,()", mid.size()) != std::string::npos)
                continue;
            std::pair<std::string, int> c{arg.substr(1), sz->second};
            if (std::find(cols.begin(), cols.end(), c) == cols.end()) cols.push_back(c);
        }
        if (cols.empty()) return false;
        src << "#define RF_PREFETCH 1\n";
        src << "RF_DEV void rf_prefetch_rows(const RfParams& P, long long r0, long long r1)\n{\n";
        for (auto& c : cols) src << "    rf_pf(" << c.first << ", r0, r1, " << c.second << ");\n";
        src << "}\n\n";
        return true;
    }

    void gen_group_reduce(std::ostringstream& src, const Reduce& red, const Drive& d, std::vector<Leaf>& leaves,
                          const std::vector<std::vector<int>>& groups, const std::vector<Expr>& key_exprs,
                          const std::vector<Expr>& filters)
    {
        plan_.kind = PlanKind::GROUP_REDUCE;
        const int T = plan_.threads;
        const int G = (int)groups.size(), M = (int)groups[0].size();
        plan_.groups = G;
        plan_.aggs = M;
        const auto& g0 = groups[0];
        std::ostringstream o;
        o << "#define RF_G " << G << "\n#define RF_M " << M << "\n\n";
        // per-aggregate value struct
        o << "struct RfVals {\n";
        for (int m = 0; m < M; m++) {
            auto& lf = leaves[g0[m]];
            std::string ct = lf.count ? "long long" : (lf.op == AggOp::OR || lf.op == AggOp::AND) ? "long long" : ctype(lf.type);
            o << "    " << ct << " v" << m << ";\n";
        }
        o << "};\n\n";
        // 64-bit slot encode/decode per aggregate
        auto enc = [&](const Leaf& lf, const std::string& x) -> std::string {
            if (!lf.count && lf.type.is_float()) return "rf_f2u((double)(" + x + "))";
            return "(unsigned long long)(long long)(" + x + ")";
        };
        auto dec = [&](const Leaf& lf, const std::string& x) -> std::string {
            if (!lf.count && lf.type.is_float()) return "rf_u2f(" + x + ")";
            if (lf.type.is_unsigned()) return "(unsigned long long)(" + x + ")";
            return "(long long)(" + x + ")";
        };
        // slot identity (sums: 0; idempotent ops: the leaf's init, per aggregate index m; the
        // init must then agree across groups, which holds for the shapes detect_groups admits
        // only when it is the same expression - checked here)
        Emitter Ei(*this);
        bind_inputs(Ei);
        std::ostringstream initsw;
        for (int m = 0; m < M; m++) {
            auto& lf = leaves[g0[m]];
            std::string v = lf.op == AggOp::SUM ? "0ULL" : enc(lf, "(" + acc_ctype(lf) + ")(" + Ei.ev(lf.init).c + ")");
            if (lf.op != AggOp::SUM)
                for (int g = 1; g < G; g++)
                    if (!same(leaves[groups[g][m]].init, lf.init)) throw LowerError("grouped min/max with differing inits");
            initsw << "        case " << m << ": return " << v << ";\n";
        }
        o << "RF_DEV unsigned long long rf_slot_init(const RfParams& P, int m)\n{\n";
        for (auto& dcl : Ei.decls) o << "    " << dcl << "\n";
        o << "    switch (m) {\n" << initsw.str() << "        default: return 0ULL;\n    }\n}\n\n";
        o << "RF_DEV unsigned long long rf_slot_combine(int m, unsigned long long a, unsigned long long b)\n{\n    switch (m) {\n";
        for (int m = 0; m < M; m++) {
            auto& lf = leaves[g0[m]];
            std::string ct = lf.count ? "long long" : (lf.op == AggOp::OR || lf.op == AggOp::AND) ? "long long" : ctype(lf.type);
            std::string A = "(" + ct + ")" + dec(lf, "a"), B = "(" + ct + ")" + dec(lf, "b");
            std::string e = combine_expr(lf, A, B);
            o << "        case " << m << ": return " << enc(lf, e) << ";\n";
        }
        o << "        default: return a;\n    }\n}\n\n";
        // FP64 SUM slots accumulate as double-floats on the FP32 pipe while `df` (the thread's
        // mode for the unit) holds, in kernels whose rows mostly reach the slots (not in a
        // compacting probe kernel: there few rows add anything, and the longer slot update costs
        // the probes occupancy - the 200M-row join measured 1.11 -> 1.23 ms with it)
        auto emit_slot_add = [&](std::ostream& so, bool use_df) {
            // an addend that is negative or out of the double-float range turns every such slot of
            // the thread into a double and the thread continues in FP64 (rf_df_step in
            // rf_device.cuh); rf_slots_done leaves doubles in all slots for the block's fold
            std::vector<int> dfm;
            for (int m = 0; m < M; m++) {
                auto& lf = leaves[g0[m]];
                if (use_df && lf.op == AggOp::SUM && !lf.count && lf.type.btype == FLOAT64) dfm.push_back(m);
            }
            if (!dfm.empty()) so << "#define RF_GROUP_UNROLL 1\n\n";
            so << "RF_DEV void rf_slots_done(unsigned long long* S, int t, bool& df)\n{\n";
            if (!dfm.empty()) {
                so << "    if (!df) return;\n    df = false;\n    for (int g = 0; g < RF_G; g++) {\n";
                for (int m : dfm)
                    so << "        { unsigned long long* s = S + (g * RF_M + " << m << ") * " << T
                      << " + t; *s = rf_df_slot_to_f64(*s); }\n";
                so << "    }\n";
            } else {
                so << "    (void)S; (void)t; (void)df;\n";
            }
            so << "}\n\n";
            so << "RF_DEV void rf_slot_add(unsigned long long* S, int g, int t, const RfVals& V, bool& df)\n{\n";
            auto slot_ptr = [&](int m) {
                return "S + (g * RF_M + " + std::to_string(m) + ") * " + std::to_string(T) + " + t";
            };
            if (!dfm.empty()) {
                // every double-float slot of the row in one pass (independent latency chains), one
                // combined check, then all stores - or the switch to FP64 for the rest of the unit
                so << "    bool fp64 = !df;\n    if (df) {\n        bool ok = true;\n";
                for (int m : dfm)
                    so << "        float2* p" << m << " = (float2*)(" << slot_ptr(m) << ");\n        float2 n" << m << ";\n";
                for (int m : dfm) so << "        ok &= rf_df_step(*p" << m << ", V.v" << m << ", n" << m << ");\n";
                so << "        if (ok) {\n";
                for (int m : dfm) so << "            *p" << m << " = n" << m << ";\n";
                so << "        } else {\n            rf_slots_done(S, t, df);\n            fp64 = true;\n        }\n    }\n";
                so << "    if (fp64) {\n";
                for (int m : dfm) {
                    auto& lf = leaves[g0[m]];
                    so << "        { unsigned long long* s = " << slot_ptr(m) << "; *s = rf_slot_combine(" << m << ", *s, "
                      << enc(lf, "V.v" + std::to_string(m)) << "); }\n";
                }
                so << "    }\n";
            }
            for (int m = 0; m < M; m++) {
                if (std::find(dfm.begin(), dfm.end(), m) != dfm.end()) continue;
                auto& lf = leaves[g0[m]];
                so << "    { unsigned long long* s = " << slot_ptr(m) << "; *s = rf_slot_combine(" << m << ", *s, "
                  << enc(lf, "V.v" + std::to_string(m)) << "); }\n";
            }
            so << "    (void)df;\n}\n\n";
        };

        // group function
        Emitter E(*this);
        std::ostringstream body;
        std::string rowcond = bind_row(E, red, d, body);
        std::ostringstream gb;
        std::string filt = "true";
        if (!filters.empty()) {
            Expr f = filters[0];
            for (size_t i = 1; i < filters.size(); i++) f = reffiner::_and(f, filters[i]);
            filt = E.ev(order_conjuncts(f)).c;
        }
        std::string gconds = filt;
        gb << "    if (!(" << filt << ")) return -1;\n";
        for (size_t k = 0; k < key_exprs.size(); k++) {
            std::string kc = E.ev(key_exprs[k]).c;
            gconds += kc;
            gb << "    const auto key" << k << " = " << kc << ";\n";
        }
        // the group whose keys match, as selects from the last group to the first (the first
        // match wins, as in an if-else chain, without a branch per group)
        gb << "    int g = -1;\n";
        for (int g = G - 1; g >= 0; g--) {
            auto& lf = leaves[groups[g][0]];
            gb << "    g = (";
            for (size_t k = 0; k < key_exprs.size(); k++) {
                if (k) gb << " && ";
                gb << "(key" << k << " == " << E.ev(lf.keys[k].second).c << ")";
            }
            gb << ") ? " << g << " : g;\n";
        }
        gb << "    if (g < 0) return -1;\n";
        for (int m = 0; m < M; m++) {
            auto& lf = leaves[g0[m]];
            std::string val;
            if (lf.count) val = "1";
            else if (lf.op == AggOp::OR || lf.op == AggOp::AND) val = "(long long)(" + E.ev(lf.value).c + ")";
            else val = "(" + ctype(lf.type) + ")(" + E.ev(lf.value).c + ")";
            gb << "    V.v" << m << " = " << val << ";\n";
        }
        gb << "    return g;\n";
        std::string gbody = gb.str();
        std::vector<std::string> dcls(E.decls.begin(), E.decls.end());
        std::vector<std::string*> pieces{&rowcond, &gbody};
        for (auto& dd : dcls) pieces.push_back(&dd);
        // The driving row's columns are read up front: the filter's, the keys', an index
        // probe's key, and - without a probe - the value columns, so that a row waits on one
        // round trip to memory (the 6-group group-by: 0.776 -> 0.667 ms with its value columns
        // read up front).  With a probe the values are read once the row has passed it: rows
        // that miss then read no value sectors, and the scan pushes less of the probed index out
        // of L2 (the 200M-row join: 1.099 ms with the probe key read inside the probe, 1.074 ms
        // (5.88 GB read) with key and value up front, 1.050 ms (4.81 GB) with the key alone)
        bool probes = gbody.find("rf_locate") != std::string::npos || rowcond.find("rf_locate") != std::string::npos;
        std::string dtext;
        for (auto& dd : dcls) {
            probes = probes || dd.find("rf_locate") != std::string::npos;
            dtext += dd;
        }
        std::string hoisted = hoist_row_loads(rowcond + gconds + dtext + (probes ? std::string() : gbody), pieces);
        if (probes) {
            const std::string mk = "    if (g < 0) return -1;\n";
            const size_t at = gbody.find(mk);
            if (at != std::string::npos) hoist_value_loads(gbody, at + mk.size());
        }
        std::ostringstream grp;
        // the row's loads as their own function (rf_group_ld into RfRowLd) and the rest
        // (rf_group_v), so that a kernel can issue the loads of several rows before it uses any
        std::vector<std::array<std::string, 3>> hl;  // type, name, load call
        if (!probes) {
            std::istringstream in(hoisted);
            std::string line;
            while (std::getline(in, line)) {
                size_t c = line.find("const "), eq = line.find(" = rf_ld<");
                if (c == std::string::npos || eq == std::string::npos || line.back() != ';') {
                    hl.clear();
                    break;
                }
                std::string decl = line.substr(c + 6, eq - c - 6);
                size_t sp = decl.rfind(' ');
                hl.push_back({decl.substr(0, sp), decl.substr(sp + 1), line.substr(eq + 3, line.size() - eq - 4)});
            }
        }
        if (!hl.empty()) {
            grp << "struct RfRowLd {\n";
            for (auto& h : hl) grp << "    " << h[0] << " " << h[1] << ";\n";
            grp << "};\n\nRF_DEV void rf_group_ld(const RfParams& P, long long r, RfRowLd& L)\n{\n";
            for (auto& h : hl) grp << "    L." << h[1] << " = " << h[2] << ";\n";
            grp << "}\n\nRF_DEV int rf_group_v(const RfParams& P, long long r, const RfRowLd& L, RfVals& V)\n{\n";
            grp << body.str();
            for (auto& h : hl) grp << "    const " << h[0] << " " << h[1] << " = L." << h[1] << ";\n";
            for (auto& dcl : dcls) grp << "    " << dcl << "\n";
            grp << "    if (!(" << rowcond << ")) return -1;\n";
            grp << gbody << "}\n\n";
            grp << "RF_DEV int rf_group(const RfParams& P, long long r, RfVals& V)\n{\n    RfRowLd L;\n"
                   "    rf_group_ld(P, r, L);\n    return rf_group_v(P, r, L, V);\n}\n\n#define RF_GROUP_SPLIT 1\n";
            // several rows a thread per loop iteration, their loads issued together: more of each
            // warp's row loads in flight.  Four for a row of up to 12 register words (the 6-group
            // group-by, 11: 0.634 ms with one row, 0.584 / 0.598 / 0.563 / 0.581 / 0.564 / 0.607
            // ms with 2 / 3 / 4 / 5 / 6 / 8, each with the tuner's tiling); wider rows take two, or
            // one past 32 words, so that the rows' values fit the registers (a group-by summing 12
            // or 14 double columns spills 124 / 220 bytes with four rows, none with two; the
            // 14-column one on 4M rows: 0.204 ms with two rows a step, 0.215 ms with one)
            int words = 0;
            for (auto& h : hl) words += (h[0] == "double" || h[0] == "int64_t" || h[0] == "uint64_t") ? 2 : 1;
            grp << "#define RF_GROUP_ROWS " << (words <= 12 ? 4 : words <= 32 ? 2 : 1) << "\n";
            grp << "\n";
        } else {
            grp << "RF_DEV int rf_group(const RfParams& P, long long r, RfVals& V)\n{\n";
            grp << body.str() << hoisted;
            for (auto& dcl : dcls) grp << "    " << dcl << "\n";
            grp << "    if (!(" << rowcond << ")) return -1;\n";
            grp << gbody << "}\n\n";
        }
        const std::string grp_text = grp.str();
        o << grp_text;
        // Rows reach an index probe (Locate) only through cheaper filter conjuncts: the kernel
        // then tests those first and queues the passing rows per warp, so each round of probes
        // runs on 32 rows at once rather than on the few lanes of a warp that passed
        // (RF_COMPACT in the template; rf_cheap is the cheap prefix of the condition).
        bool compact = false;
        {
            std::string fn_text = body.str() + hoisted + gbody;
            for (auto& dcl : dcls) fn_text += dcl;
            std::vector<Expr> cheap;
            if (!filters.empty() && fn_text.find("rf_locate") != std::string::npos) {
                Expr f = filters[0];
                for (size_t i = 1; i < filters.size(); i++) f = reffiner::_and(f, filters[i]);
                std::vector<Expr> cj;
                flatten_and(order_conjuncts(f), cj);
                for (auto& c : cj) {
                    if (cost_of(c) >= 20) break;
                    cheap.push_back(c);
                }
            }
            if (!cheap.empty()) {
                compact = true;
                Emitter Ec(*this);
                std::ostringstream cbody;
                std::string crow = bind_row(Ec, red, d, cbody);
                Expr cf = cheap[0];
                for (size_t i = 1; i < cheap.size(); i++) cf = reffiner::_and(cf, cheap[i]);
                std::string cc = Ec.ev(cf).c;
                std::vector<std::string> cd(Ec.decls.begin(), Ec.decls.end());
                std::string cret = "    return " + cc + ";\n";
                std::vector<std::string*> cp{&crow, &cret};
                for (auto& x : cd) cp.push_back(&x);
                std::string ch = hoist_row_loads(crow + cc, cp);
                o << "RF_DEV bool rf_cheap(const RfParams& P, long long r)\n{\n" << cbody.str() << ch;
                for (auto& x : cd) o << "    " << x << "\n";
                o << "    if (!(" << crow << ")) return false;\n" << cret << "}\n\n#define RF_COMPACT 1\n\n";
            }
        }

        emit_slot_add(o, !compact);
        push_index_filter(o, red, filters);
        // A grouped scan that reads every row's columns prefetches the next tile into L2 while it
        // works on this one (the 60M-row, 6-group group-by: 1.23 -> 1.15 ms; its FP64 work waited
        // on DRAM loads).  A compacting one reads most columns only for the rows that pass its
        // cheap test (the 200M-row join's probe scan measured 1.45 -> 1.70 ms with a prefetch: it
        // needs L2 for its filtered index), and a one-tile filter+sum unit measured slower with its
        // own tile prefetched (0.048 -> 0.052 ms).
        if (!compact && d.input >= 0 && d.slot >= 0) emit_prefetch(o, grp_text, d.slot);

        // epilogue
        Emitter Ef(*this);
        bind_inputs(Ef);
        std::map<std::vector<size_t>, std::string> finals;
        std::ostringstream fb;
        std::map<int, std::pair<int, int>> leaf_gm;
        for (int g = 0; g < G; g++)
            for (int m = 0; m < M; m++) leaf_gm[groups[g][m]] = {g, m};
        for (size_t i = 0; i < leaves.size(); i++) {
            auto& lf = leaves[i];
            std::string tot = "0";
            if (lf.op != AggOp::NONE) {
                auto gm = leaf_gm.at((int)i);
                tot = dec(lf, "S[" + std::to_string(gm.first * M + gm.second) + "]");
            }
            std::string nm = "st" + std::to_string(i);
            fb << "    const " << ctype(lf.type) << " " << nm << " = " << final_leaf(Ef, lf, tot) << ";\n";
            finals[lf.path] = nm;
        }
        std::ostringstream stores;
        emit_output_store(Ef, stores, red, finals);
        o << "RF_DEV void rf_finish_groups(const RfParams& P, const unsigned long long* S, unsigned char* out)\n{\n";
        for (auto& dcl : Ef.decls) o << "    " << dcl << "\n";
        o << fb.str() << stores.str() << "}\n\n";

        src << o.str();
        size_t smem = (size_t)G * M * T * 8 + (compact ? (size_t)(T / 32) * 64 * 8 : 0);
        if (smem > 200 * 1024) throw LowerError("too many group accumulators for shared memory");
        // the blocks an SM holds by shared memory (228 KiB, 1 KiB reserved per block) are the
        // blocks the registers should allow too, so the compiler is asked to fit that many - down
        // to 80 registers a thread (the double-float slot update of the 6-group group-by needs
        // about that many; a compacting probe kernel keeps the compiler's own choice)
        const int minb = compact ? 1
                                 : (int)std::max<size_t>(1, std::min<size_t>({(size_t)2048 / T, (228 * 1024) / (smem + 1024),
                                                                              (size_t)65536 / (80 * (size_t)T)}));
        src << "#define RF_GROUP_REDUCE 1\n";
        if (minb > 1) src << "#define RF_MINB " << minb << "\n";
        src << "#include \"rf_templates.cuh\"\n";
        src << "RF_GROUP_REDUCE_KERNEL(rf_main, " << T << ")\n";
        plan_.kernels.push_back({"rf_main", T, smem, KernelSpec::MAIN});
        plan_.acc_bytes = (size_t)G * M * 8;
    }

    // ---------------------------------------------------------------- Op lowering (tables)
    // binds the Op's iterator for element r of its iteration space; returns the element's
    // iteration condition (VecSpace: r < len && valid(col0, r); bounds; filter symbols)
    std::string bind_op_row(Emitter& E, const Op& op, const Drive& d, std::ostringstream& body)
    {
        const Space& sp = d.sp;
        std::string T = ctype(sp.iter->type);
        std::string sl = std::to_string(d.slot);
        std::string it_c, cond;
        if (sp.has_vec) {
            note_col(d.input, 0);
            it_c = "rf_ld<" + T + ">(P.t[" + sl + "].col[0].data, r)";
            cond = "rf_valid(P.t[" + sl + "].col[0].valid, r)";
            E.vec_iter_idx[{sp.vec_node.get(), sp.iter.get()}] = "r";
        } else {
            it_c = "((" + T + ")r)";
            cond = "true";
        }
        body << "    const " << T << " it = " << it_c << ";\n";
        E.bind(op.iters[0], E.scalar("it", sp.iter->type));
        if (!sp.lbs.empty()) cond += " && (it >= (" + T + ")P.range[2])";
        if (!sp.ubs.empty()) cond += " && (it <= (" + T + ")P.range[3])";
        for (auto& f : sp.filters) cond += " && (" + E.ev(f).c + ")";
        return cond;
    }

    void drive_rows(Drive& d)
    {
        if (d.sp.has_vec) {
            d.input = d.sp.vec_input;
            d.slot = plan_.table_slot[d.input];
            plan_.drive_input = d.input;
            HostExpr lo;
            lo.kind = HostExpr::CONST;
            lo.value = 0;
            HostExpr hi;
            hi.kind = HostExpr::LEN;
            hi.input = d.input;
            hi.col = 0;
            plan_.row_lo = lo;
            plan_.row_hi = hi;
        } else {
            plan_.row_lo = minmax_host(d.sp.lbs, true);
            HostExpr hi = minmax_host(d.sp.ubs, false);
            HostExpr one;
            one.kind = HostExpr::CONST;
            one.value = 1;
            HostExpr h2;
            h2.kind = HostExpr::ADD;
            h2.args = {hi, one};
            plan_.row_hi = h2;
        }
    }

    // Segmented reduce over run-end encoded rows: every run is cut into chunks of RF_SEG_CH rows
    // (long Zipf runs spread over many threads); chunk c of run r is reduced by one thread in row
    // order into partial[woff[r] + c]; the element functions fold a run's partials in order.
    // woff: (long long*)P.aux4 (nruns + 1 entries), partials: (RfAcc*)P.aux5.
    void emit_seg_kernels(std::ostringstream& o, const Drive& d)
    {
        std::string c0 = "P.t[" + std::to_string(d.slot) + "].col[0]";
        o << "#define RF_SEG_CH 256\n";
        o << "extern \"C\" __global__ void __launch_bounds__(256) rf_seg_count(const __grid_constant__ RfParams P)\n{\n";
        o << "    long long* woff = (long long*)P.aux4;\n    const long long n = " << c0 << ".len;\n";
        o << "    for (long long run = blockIdx.x * (long long)blockDim.x + threadIdx.x; run < n; run += (long long)gridDim.x * blockDim.x) {\n";
        o << "        long long len = rf_runend(" << c0 << ", run) - rf_runend(" << c0 << ", run - 1);\n";
        o << "        long long c = (len + RF_SEG_CH - 1) / RF_SEG_CH;\n        woff[run] = c < 1 ? 1 : c;\n    }\n}\n\n";
        o << "extern \"C\" __global__ void __launch_bounds__(256) rf_seg_reduce(const __grid_constant__ RfParams P)\n{\n";
        o << "    const long long* woff = (const long long*)P.aux4;\n    RfAcc* part = (RfAcc*)P.aux5;\n";
        o << "    const long long n = " << c0 << ".len, W = woff[n];\n";
        o << "    for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < W; w += (long long)gridDim.x * blockDim.x) {\n";
        o << "        long long lo = 0, hi = n;  // last run with woff[run] <= w\n";
        o << "        while (hi - lo > 1) { long long mid = (lo + hi) >> 1; if (woff[mid] <= w) lo = mid; else hi = mid; }\n";
        o << "        const long long run = lo, k = w - woff[run];\n";
        o << "        const long long s = rf_runend(" << c0 << ", run - 1) + k * RF_SEG_CH;\n";
        o << "        long long e = rf_runend(" << c0 << ", run);\n        if (e > s + RF_SEG_CH) e = s + RF_SEG_CH;\n";
        o << "        RfAcc A;\n        rf_acc_init(P, A);\n        for (long long r = s; r < e; r++) rf_row(P, r, A);\n";
        o << "        rf_st_words(part + w, &A, (int)sizeof(RfAcc));\n    }\n}\n\n";
        o << "RF_DEV void rf_fold(const RfParams& P, long long run, RfAcc& A)\n{\n";
        o << "    const long long* woff = (const long long*)P.aux4;\n    const RfAcc* part = (const RfAcc*)P.aux5;\n";
        o << "    rf_acc_init(P, A);\n    for (long long w = woff[run]; w < woff[run + 1]; w++) {\n";
        o << "        RfAcc p;\n        rf_ld_words(&p, part + w, (int)sizeof(RfAcc));\n        rf_acc_combine(A, p);\n    }\n}\n\n";
        plan_.kernels.push_back({"rf_seg_count", 256, 0, KernelSpec::SEGCOUNT});
        plan_.kernels.push_back({"", 0, 0, KernelSpec::SEGSCAN});
        plan_.kernels.push_back({"rf_seg_reduce", 256, 0, KernelSpec::SEGREDUCE});
    }

    // the final state of a folded accumulator `SA`, as a struct value
    Val seg_state(Emitter& E, std::ostringstream& body, const Reduce& red, std::vector<Leaf>& leaves)
    {
        std::map<std::vector<size_t>, std::string> finals;
        for (size_t i = 0, k = 0; i < leaves.size(); i++) {
            auto& lf = leaves[i];
            std::string tot = lf.op == AggOp::NONE ? "0" : "SA.a" + std::to_string(k++);
            std::string nm = "sst" + std::to_string(i);
            body << "    const " << ctype(lf.type) << " " << nm << " = " << final_leaf(E, lf, tot) << ";\n";
            finals[lf.path] = nm;
        }
        std::function<Val(const DataType&, std::vector<size_t>)> mk = [&](const DataType& t, std::vector<size_t> pth) {
            Val v;
            v.type = t;
            if (t.is_struct()) {
                v.k = Val::STRUCT;
                for (size_t i = 0; i < t.dtypes.size(); i++) {
                    auto q = pth;
                    q.push_back(i);
                    v.f.push_back(mk(t.dtypes[i], q));
                }
                return v;
            }
            v.c = finals.at(pth);
            return v;
        };
        return mk(red.type, {});
    }

    // Hash group-by: the grouped Op over a 2-d vector whose key column (column 0) is flat and
    // unsorted.  The groups are the distinct valid keys - the runs the reference would see after
    // sorting and run-end encoding - so each output row is the same; rows come out in slot order.
    //   rf_hg_init  fills the table: keys RF_EMPTY_KEY, accumulators at their identity
    //   rf_hg_agg   one pass over the rows.  A per-block shared-memory table takes the keys a
    //               block meets first - under a skewed distribution the frequent ones - and
    //               absorbs their updates with shared-memory atomics; a key found neither there
    //               nor in a free shared slot goes to the global open-addressing table (load 0.5)
    //   rf_cond / rf_emit   the materialisation template over the slots
    // Global slots are array-of-structs, {key, accumulators...} padded to RF_HG_SW 8-byte words
    // (one 32-byte sector for up to three accumulators), so a row touches one sector.
    // Device layout: slots (unsigned long long*)P.aux4 [C + 1][RF_HG_SW] (slot C: the key
    // RF_EMPTY_KEY itself, a used flag in its key word), rows P.aux_n0, capacity C = P.aux_n1.
    // rows per lane in one step of the aggregation loop: with 2 or 4 (all loads and probes of a
    // step issued before any is used) the 100M-row group-by took 3.6 and 5.0 ms against 2.1 ms
    static int hg_rows_per_step() { return 1; }

    void lower_hash_group(const Op& op, const Drive& d, const Reduce& red)
    {
        plan_.kind = PlanKind::HASH_GROUP;
        const int T = plan_.threads;
        std::vector<Leaf> leaves;
        collect_leaves(red, red.type, {}, leaves);
        std::vector<int> act;
        for (size_t i = 0; i < leaves.size(); i++)
            if (leaves[i].op != AggOp::NONE) act.push_back((int)i);
        const int L = (int)act.size();
        // shared-memory tiers of the aggregation kernel (see rf_hg_agg below): HK hottest keys
        // with warp-private accumulators, WK further hot keys with block-shared accumulators
        // the aggregation kernel's hottest keys (see rf_hg_agg below): HK keys with warp-private
        // accumulators, at most 16 KB of them per block
        const int HT = 256, HW = HT / 32, LL = std::max(L, 1);
        int HK = 128;
        while (HK > 8 && HW * HK * LL * 8 > 16 * 1024) HK /= 2;
        plan_.hg_hot = HK;
        plan_.hg_warm = 0;
        std::string sl = std::to_string(d.slot);
        std::string c0 = "P.t[" + sl + "].col[0]";
        std::ostringstream o;
        o << "// generated by the reffine_gb300 lowering pass: " << fn_->name << " (hash group-by)\n";
        const int SW = L + 1 <= 4 ? 4 : (L + 1 <= 8 ? 8 : 16);
        if (L + 1 > 16) throw LowerError("hash group-by with more than 15 aggregates");
        o << "#include \"rf_device.cuh\"\n\n#define RF_HG_L " << LL << "\n#define RF_HG_SW " << SW
          << "\n#define RF_HG_T " << HT << "\n#define RF_HG_HK " << HK << "\n#define RF_HG_U " << hg_rows_per_step()
          << "\n#define RF_HG_SPK " << kHotSlotsPerKey << "\n\n";
        plan_.acc_bytes = (size_t)SW * 8;
        auto kind_of = [&](const Leaf& lf) -> std::string {
            bool f = lf.type.is_float() && !lf.count;
            switch (lf.op) {
                case AggOp::SUM: return f ? "fsum" : "isum";
                case AggOp::MAX: return f ? "fmax" : (lf.type.is_unsigned() ? "umax" : "imax");
                case AggOp::MIN: return f ? "fmin" : (lf.type.is_unsigned() ? "umin" : "imin");
                case AggOp::OR: return "or";
                case AggOp::AND: return "and";
                default: return "none";
            }
        };
        auto enc = [&](const Leaf& lf, const std::string& x) -> std::string {
            if (lf.type.is_float() && !lf.count) return "rf_f2u((double)(" + x + "))";
            return "(unsigned long long)(long long)(" + x + ")";
        };
        auto arg = [&](const Leaf& lf, const std::string& raw) -> std::string {
            if (lf.type.is_float() && !lf.count) return "rf_u2f(" + raw + ")";
            if (kind_of(lf) == "umax" || kind_of(lf) == "umin") return raw;
            return "(long long)(" + raw + ")";
        };
        // identities
        {
            Emitter Ei(*this);
            bind_inputs(Ei);
            std::ostringstream b;
            for (int k = 0; k < L; k++) {
                auto& lf = leaves[act[k]];
                std::string v = lf.op == AggOp::SUM ? "0ULL" : enc(lf, "(" + acc_ctype(lf) + ")(" + Ei.ev(lf.init).c + ")");
                b << "    case " << k << ": return " << v << ";\n";
            }
            o << "RF_DEV unsigned long long rf_hg_identity(const RfParams& P, int l)\n{\n";
            for (auto& dcl : Ei.decls) o << "    " << dcl << "\n";
            o << "    switch (l) {\n" << b.str() << "    default: return 0ULL;\n    }\n}\n\n";
        }
        // One row's contribution: the columns it reads are loaded first into a row struct
        // (rf_hg_load, so a thread issues the loads of several rows before using any of them),
        // then added to a slot's accumulators (rf_hg_apply: slot A, leaf stride `st`, atomics) or
        // returned as values (rf_hg_vals: the identity where the row adds nothing, for the
        // warp-level fold of the hottest keys).
        {
            const DataType& vt = fn_->inputs[d.input]->type;
            auto bind_row_struct = [&](Emitter& E) {
                Val v;
                v.k = Val::STRUCT;
                v.type = red.val->type;
                for (size_t c = 1; c < vt.dtypes.size(); c++) v.f.push_back(E.scalar("R.v" + std::to_string(c), vt.dtypes[c]));
                E.bind(red.val, v);
            };
            Emitter E(*this);
            bind_inputs(E);
            bind_row_struct(E);
            std::ostringstream u, xv;
            for (int k = 0; k < L; k++) {
                auto& lf = leaves[act[k]];
                std::string cond = lf.cond ? E.ev(order_conjuncts(lf.cond)).c : "";
                std::string val = lf.count ? "1" : "(" + acc_ctype(lf) + ")(" + E.ev(lf.value).c + ")";
                std::string call = "rf_atom_" + kind_of(lf) + "(A + " + std::to_string(k) + " * st, " + val + ")";
                if (kind_of(lf) == "fmax" || kind_of(lf) == "fmin") call = "if (!" + call + ") rf_set_err(P, RF_DEVERR_WAIT)";
                if (!cond.empty()) u << "    if (" << cond << ") { " << call << "; }\n";
                else u << "    " << call << ";\n";
                std::string x = enc(lf, val);
                if (!cond.empty()) xv << "    x[" << k << "] = (" << cond << ") ? " << x << " : rf_hg_identity(P, " << k << ");\n";
                else xv << "    x[" << k << "] = " << x << ";\n";
            }
            std::string body = u.str() + xv.str();
            for (auto& dcl : E.decls) body += dcl;
            // the row struct holds exactly the columns the contribution reads
            o << "struct RfHgRow {\n    bool ok;\n";
            std::ostringstream ld;
            ld << "RF_DEV void rf_hg_load(const RfParams& P, long long r, RfHgRow& R)\n{\n";
            ld << "    R.ok = rf_valid(P.t[" << sl << "].col[1].valid, r);  // loopgen.cpp:238\n";
            for (size_t c = 1; c < vt.dtypes.size(); c++) {
                std::string f = "R.v" + std::to_string(c);
                bool used = false;
                for (size_t pos = body.find(f); pos != std::string::npos; pos = body.find(f, pos + 1)) {
                    char nx = pos + f.size() < body.size() ? body[pos + f.size()] : ' ';
                    if (!isdigit((unsigned char)nx)) used = true;
                }
                if (!used) continue;
                o << "    " << ctype(vt.dtypes[c]) << " v" << c << ";\n";
                ld << "    " << f << " = rf_ld<" << ctype(vt.dtypes[c]) << ">(P.t[" << sl << "].col[" << c << "].data, r);\n";
            }
            o << "};\n\n" << ld.str() << "}\n\n";
            o << "RF_DEV void rf_hg_apply(const RfParams& P, const RfHgRow& R, unsigned long long* A, long long st)\n{\n";
            o << "    if (!R.ok) return;\n";
            for (auto& dcl : E.decls) o << "    " << dcl << "\n";
            o << u.str() << "    (void)A; (void)st;\n}\n\n";
            o << "RF_DEV void rf_hg_vals(const RfParams& P, const RfHgRow& R, unsigned long long* x)\n{\n";
            o << "    if (!R.ok) {\n        for (int l = 0; l < RF_HG_L; l++) x[l] = rf_hg_identity(P, l);\n        return;\n    }\n";
            for (auto& dcl : E.decls) o << "    " << dcl << "\n";
            o << xv.str() << "}\n\n";
            o << "RF_DEV unsigned long long rf_hg_comb(int l, unsigned long long a, unsigned long long b)\n{\n    switch (l) {\n";
            for (int k = 0; k < L; k++) {
                auto& lf = leaves[act[k]];
                std::string ct = lf.count ? "long long"
                                 : (lf.op == AggOp::OR || lf.op == AggOp::AND) ? "long long" : acc_ctype(lf);
                bool f = lf.type.is_float() && !lf.count;
                std::string A = f ? "rf_u2f(a)" : "(" + ct + ")(a)", B = f ? "rf_u2f(b)" : "(" + ct + ")(b)";
                o << "        case " << k << ": return " << enc(lf, combine_expr(lf, A, B)) << ";\n";
            }
            o << "        default: return a;\n    }\n}\n\n";
        }
        // flush of a pre-aggregated slot into the global table
        o << "RF_DEV void rf_hg_merge(const RfParams& P, unsigned long long* A, long long st, const unsigned long long* B, long long bst)\n{\n";
        for (int k = 0; k < L; k++) {
            auto& lf = leaves[act[k]];
            std::string raw = "B[" + std::to_string(k) + " * bst]";
            std::string call = "rf_atom_" + kind_of(lf) + "(A + " + std::to_string(k) + " * st, " + arg(lf, raw) + ")";
            if (kind_of(lf) == "fmax" || kind_of(lf) == "fmin") call = "if (!" + call + ") rf_set_err(P, RF_DEVERR_WAIT)";
            o << "    " << call << ";\n";
        }
        o << "    (void)A; (void)B; (void)st; (void)bst;\n}\n\n";
        o << R"(// slot of `key` in the global table from probe position h on (claimed if new): one
// compare-and-swap per probe, which claims an empty slot or finds the key in one round trip
// (hot keys never come here, so the slots are not contended)
RF_DEV long long rf_hg_slot_from(const RfParams& P, long long key, unsigned long long h, unsigned long long n0)
{
    unsigned long long* tab = (unsigned long long*)P.aux4;
    const unsigned long long C = (unsigned long long)P.aux_n1;
    for (unsigned long long n = 0; n < n0; ++n) {
        const unsigned long long old =
            atomicCAS(tab + h * RF_HG_SW, (unsigned long long)RF_EMPTY_KEY, (unsigned long long)key);
        if (old == (unsigned long long)RF_EMPTY_KEY || old == (unsigned long long)key) return (long long)h;
        if (++h == C) h = 0;
    }
    rf_set_err(P, RF_DEVERR_OVERFLOW);
    return -1;
}

// slot of `key` in the global table (claimed if new); C + 1 slots, slot C is the empty key's
RF_DEV long long rf_hg_slot(const RfParams& P, long long key)
{
    unsigned long long* tab = (unsigned long long*)P.aux4;
    const unsigned long long C = (unsigned long long)P.aux_n1;
    if (key == RF_EMPTY_KEY) {
        if (tab[C * RF_HG_SW] == 0) atomicExch(tab + C * RF_HG_SW, 1ULL);
        return (long long)C;
    }
    return rf_hg_slot_from(P, key, rf_home(key, C), C);
}

extern "C" __global__ void __launch_bounds__(256) rf_hg_init(const __grid_constant__ RfParams P)
{
    unsigned long long* tab = (unsigned long long*)P.aux4;
    const long long C = P.aux_n1;
    // word by word, so a warp's stores are contiguous
    const long long words = (C + 1) * RF_HG_SW;
    for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < words; w += (long long)gridDim.x * blockDim.x) {
        const long long s = w / RF_HG_SW;
        const int f = (int)(w % RF_HG_SW);
        tab[w] = f == 0 ? (s < C ? (unsigned long long)RF_EMPTY_KEY : 0ULL)
                        : (f <= RF_HG_L ? rf_hg_identity(P, f - 1) : 0ULL);
    }
}

// Aggregation.  Rows of the hottest keys (chosen from a sample of the key column, so Zipf-like
// skew lands here) fold inside each warp: the lanes holding the same hot key find each other
// with __match_any_sync, the lowest of them folds their contributions and adds them, without
// atomics, to the warp's own accumulators.  All other rows go to the global table, whose
// accumulators take fire-and-forget atomics; its keys are read through L1 first (a claimed
// slot's key never changes; a stale empty is corrected by the compare-and-swap).  The hot-key
// index is a read-only table built on the host: open addressing, load <= 0.5, 32-bit
// multiplicative hash of the folded key.
// The hot-key table is collision-free (the host chose its hash multiplier and left out any key
// whose slot a hotter key took), so a lookup is one probe.
// Dynamic shared memory:
//   hk[HKS] i64 | hid[HKS] u8 | wacc[W][HK][L] | xs[W][32][L] | seen[HK] u8,  HKS = RF_HG_SPK * HK
// (a key is a group as soon as one valid row has it, whatever the row adds)
RF_DEV unsigned rf_hg_h32(long long key, unsigned mult, int bits)
{
    const unsigned f = (unsigned)key ^ (unsigned)((unsigned long long)key >> 32);
    return (f * mult) >> (32 - bits);
}

RF_DEV long long rf_hg_slot_l1(const RfParams& P, long long key, unsigned long long h, unsigned long long n0)
{
    unsigned long long* tab = (unsigned long long*)P.aux4;
    const unsigned long long C = (unsigned long long)P.aux_n1;
    for (unsigned long long n = 0; n < n0; ++n) {
        unsigned long long* kp = tab + h * RF_HG_SW;
        const unsigned long long cur = __ldca(kp);
        if (cur == (unsigned long long)key) return (long long)h;
        if (cur == (unsigned long long)RF_EMPTY_KEY) {
            const unsigned long long old = atomicCAS(kp, (unsigned long long)RF_EMPTY_KEY, (unsigned long long)key);
            if (old == (unsigned long long)RF_EMPTY_KEY || old == (unsigned long long)key) return (long long)h;
        }
        if (++h == C) h = 0;
    }
    rf_set_err(P, RF_DEVERR_OVERFLOW);
    return -1;
}

extern "C" __global__ void __launch_bounds__(RF_HG_T) rf_hg_agg(const __grid_constant__ RfParams P)
{
    constexpr int W = RF_HG_T / 32, HKS = RF_HG_SPK * RF_HG_HK;
    int bits = 0;
    while ((1 << bits) < HKS) bits++;
    extern __shared__ __align__(16) unsigned char smem[];
    long long* hk = (long long*)smem;
    unsigned char* hid = (unsigned char*)(hk + HKS);
    unsigned long long* wacc = (unsigned long long*)(smem + ((size_t)HKS * 9 + 15) / 16 * 16);
    unsigned long long* xs = wacc + (size_t)W * RF_HG_HK * RF_HG_L;
    unsigned char* seen = (unsigned char*)(xs + (size_t)W * 32 * RF_HG_L);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // the hot-key image: multiplier | hk | hid (aux5; null: no hot keys)
    const unsigned char* img = (const unsigned char*)P.aux5;
    const unsigned mult = img ? *(const unsigned*)img : 0x9E3779B1u;
    for (int i = tid; i < HKS; i += RF_HG_T) {
        hk[i] = img ? ((const long long*)(img + 8))[i] : RF_EMPTY_KEY;
        hid[i] = img ? img[8 + (size_t)HKS * 8 + i] : 0;
    }
    for (int i = tid; i < W * RF_HG_HK * RF_HG_L; i += RF_HG_T) wacc[i] = rf_hg_identity(P, i % RF_HG_L);
    for (int i = tid; i < RF_HG_HK; i += RF_HG_T) seen[i] = 0;
    __syncthreads();
    unsigned long long* tab = (unsigned long long*)P.aux4;
    unsigned long long* wa = wacc + (size_t)warp * RF_HG_HK * RF_HG_L;
    unsigned long long* x = xs + ((size_t)warp * 32 + lane) * RF_HG_L;
    unsigned long long top[RF_HG_L];  // the lane's sums of hot id 0
#pragma unroll
    for (int l = 0; l < RF_HG_L; l++) top[l] = rf_hg_identity(P, l);
    bool top_seen = false;
    const long long n = P.aux_n0;
    const unsigned long long C = (unsigned long long)P.aux_n1;
    // whole warps step together (the fold needs every lane); rows past the end are inactive.  A
    // step takes RF_HG_U rows per lane (RF_HG_U x 32 consecutive rows per warp): all their loads
    // are issued first, then the hot-key probes, then the first global-table read of every cold
    // row, and only then is any of it used - the latencies overlap instead of forming one chain
    // per row
    const long long wstride = (long long)gridDim.x * RF_HG_T * RF_HG_U;
    for (long long base = ((long long)blockIdx.x * W + warp) * 32 * RF_HG_U; base < n; base += wstride) {
        bool act[RF_HG_U];
        long long key[RF_HG_U];
        RfHgRow row[RF_HG_U];
#pragma unroll
        for (int j = 0; j < RF_HG_U; j++) {
            const long long r = base + 32 * j + lane;
)";
        o << "            act[j] = r < n && rf_valid(" << c0 << ".valid, r);  // a null key is no group\n";
        o << "            key[j] = act[j] ? rf_ld<int64_t>(" << c0 << ".data, r) : RF_EMPTY_KEY;\n";
        o << R"(            if (act[j]) rf_hg_load(P, r, row[j]);
        }
        int h[RF_HG_U];
#pragma unroll
        for (int j = 0; j < RF_HG_U; j++) {
            const unsigned q = rf_hg_h32(key[j], mult, bits);
            h[j] = act[j] && key[j] != RF_EMPTY_KEY && hk[q] == key[j] ? (int)hid[q] : -1;
        }
        // first read of each cold row's home slot, issued for all the step's rows at once
        unsigned long long home[RF_HG_U], first[RF_HG_U];
#pragma unroll
        for (int j = 0; j < RF_HG_U; j++) {
            home[j] = 0;
            first[j] = (unsigned long long)RF_EMPTY_KEY;
            if (act[j] && h[j] < 0 && key[j] != RF_EMPTY_KEY) {
                home[j] = rf_home(key[j], C);
                first[j] = __ldca(tab + home[j] * RF_HG_SW);
            }
        }
#pragma unroll
        for (int j = 0; j < RF_HG_U; j++) {
            // the hottest key (hot id 0, about a tenth of the rows under Zipf(1.1)) adds into the
            // lane's own registers: no fold, and the other hot keys' folds stay short
            if (h[j] == 0) {
                unsigned long long xr[RF_HG_L];
                rf_hg_vals(P, row[j], xr);
#pragma unroll
                for (int l = 0; l < RF_HG_L; l++) top[l] = rf_hg_comb(l, top[l], xr[l]);
                top_seen = true;
            }
            // fold of the other hottest keys: lanes of one hot key find each other, the lowest
            // folds; a key alone in the warp adds straight into the warp's accumulators
            const unsigned peers = __match_any_sync(0xffffffffu, h[j] >= 1 ? h[j] : -1 - lane);
            if (h[j] >= 1 && peers == (1u << lane)) {
                unsigned long long xr[RF_HG_L];
                rf_hg_vals(P, row[j], xr);
                unsigned long long* A = wa + (size_t)h[j] * RF_HG_L;
#pragma unroll
                for (int l = 0; l < RF_HG_L; l++) A[l] = rf_hg_comb(l, A[l], xr[l]);
                seen[h[j]] = 1;
            } else if (h[j] >= 1) {
                rf_hg_vals(P, row[j], x);
                __syncwarp(peers);
                if (lane == __ffs(peers) - 1) {
                    unsigned long long a[RF_HG_L];
#pragma unroll
                    for (int l = 0; l < RF_HG_L; l++) a[l] = x[l];
                    for (unsigned m = peers & (peers - 1); m; m &= m - 1) {
                        const unsigned long long* y = xs + ((size_t)warp * 32 + (__ffs(m) - 1)) * RF_HG_L;
#pragma unroll
                        for (int l = 0; l < RF_HG_L; l++) a[l] = rf_hg_comb(l, a[l], y[l]);
                    }
                    unsigned long long* A = wa + (size_t)h[j] * RF_HG_L;
#pragma unroll
                    for (int l = 0; l < RF_HG_L; l++) A[l] = rf_hg_comb(l, A[l], a[l]);
                    seen[h[j]] = 1;
                }
                __syncwarp(peers);
            }
        }
#pragma unroll
        for (int j = 0; j < RF_HG_U; j++) {
            if (!act[j] || h[j] >= 0) continue;
            long long g;
            if (key[j] == RF_EMPTY_KEY) {
                g = rf_hg_slot(P, key[j]);
            } else if (first[j] == (unsigned long long)key[j]) {
                g = (long long)home[j];
            } else {
                // the home slot is empty (claim it) or holds another key: probe on from the next
                g = -1;
                if (first[j] == (unsigned long long)RF_EMPTY_KEY) {
                    const unsigned long long old = atomicCAS(tab + home[j] * RF_HG_SW, (unsigned long long)RF_EMPTY_KEY,
                                                             (unsigned long long)key[j]);
                    if (old == (unsigned long long)RF_EMPTY_KEY || old == (unsigned long long)key[j]) g = (long long)home[j];
                }
                if (g < 0) g = rf_hg_slot_l1(P, key[j], home[j] + 1 == C ? 0 : home[j] + 1, C - 1);
            }
            if (g >= 0) rf_hg_apply(P, row[j], tab + g * RF_HG_SW + 1, 1);
        }
    }
    // the lanes' sums of hot id 0 into their warp's accumulator of it
    if (__any_sync(0xffffffffu, top_seen)) {
#pragma unroll
        for (int l = 0; l < RF_HG_L; l++) {
            unsigned long long v = top[l];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) v = rf_hg_comb(l, v, __shfl_down_sync(0xffffffffu, v, off));
            if (lane == 0) wa[l] = rf_hg_comb(l, wa[l], v);
        }
        if (lane == 0) seen[0] = 1;
    }
    __syncthreads();
    // warp accumulators of each hottest key, folded over the warps, then into the global table
    for (int i = tid; i < HKS; i += RF_HG_T) {
        if (hk[i] == RF_EMPTY_KEY) continue;
        const int id = hid[i];
        if (!seen[id]) continue;
        unsigned long long a[RF_HG_L];
#pragma unroll
        for (int l = 0; l < RF_HG_L; l++) a[l] = wacc[(size_t)id * RF_HG_L + l];
        for (int w2 = 1; w2 < W; w2++)
#pragma unroll
            for (int l = 0; l < RF_HG_L; l++) a[l] = rf_hg_comb(l, a[l], wacc[((size_t)w2 * RF_HG_HK + id) * RF_HG_L + l]);
        const long long g = rf_hg_slot(P, hk[i]);
        if (g >= 0) rf_hg_merge(P, tab + g * RF_HG_SW + 1, 1, a, 1);
    }
}

)";
        // element functions over the slots
        auto elem = [&](Emitter& E, std::ostringstream& body) {
            body << "    const unsigned long long* sl = (const unsigned long long*)P.aux4 + r * RF_HG_SW;\n";
            body << "    const long long C = P.aux_n1;\n";
            body << "    const bool used = r < C ? (long long)sl[0] != RF_EMPTY_KEY : sl[0] != 0;\n";
            body << "    const int64_t it = r < C ? (long long)sl[0] : RF_EMPTY_KEY;\n";
            E.bind(op.iters[0], E.scalar("it", d.sp.iter->type));
            std::map<std::vector<size_t>, std::string> finals;
            for (size_t i = 0, k = 0; i < leaves.size(); i++) {
                auto& lf = leaves[i];
                std::string tot = "0";
                if (lf.op != AggOp::NONE) {
                    std::string raw = "sl[" + std::to_string(k + 1) + "]";
                    tot = (lf.type.is_float() && !lf.count) ? "rf_u2f(" + raw + ")" : "(long long)(" + raw + ")";
                    k++;
                }
                std::string nm = "hst" + std::to_string(i);
                body << "    const " << ctype(lf.type) << " " << nm << " = " << final_leaf(E, lf, tot) << ";\n";
                finals[lf.path] = nm;
            }
            std::function<Val(const DataType&, std::vector<size_t>)> mk = [&](const DataType& t, std::vector<size_t> pth) {
                Val v;
                v.type = t;
                if (t.is_struct()) {
                    v.k = Val::STRUCT;
                    for (size_t i = 0; i < t.dtypes.size(); i++) {
                        auto q = pth;
                        q.push_back(i);
                        v.f.push_back(mk(t.dtypes[i], q));
                    }
                    return v;
                }
                v.c = finals.at(pth);
                return v;
            };
            E.node_bind[(const ExprNode*)&red] = mk(red.type, {});
        };
        {
            Emitter E(*this);
            bind_inputs(E);
            std::ostringstream body;
            elem(E, body);
            std::string cond = "used";
            for (auto& lb : d.sp.lbs) cond += " && (it >= (int64_t)(" + E.ev(lb).c + "))";
            for (auto& ub : d.sp.ubs) cond += " && (it <= (int64_t)(" + E.ev(ub).c + "))";
            for (auto& f : d.sp.filters) cond += " && (" + E.ev(f).c + ")";
            o << "RF_DEV bool rf_cond(const RfParams& P, long long r)\n{\n" << body.str();
            for (auto& dcl : E.decls) o << "    " << dcl << "\n";
            o << "    return " << cond << ";\n}\n\n";
        }
        {
            Emitter E(*this);
            bind_inputs(E);
            std::ostringstream body;
            elem(E, body);
            std::ostringstream w;
            size_t c = 0;
            w << "    ((int64_t*)((void* const*)P.aux0)[" << c++ << "])[o] = it;\n";
            for (auto& x : op.outputs) {
                w << "    ((" << ctype(x->type) << "*)((void* const*)P.aux0)[" << c << "])[o] = (" << ctype(x->type) << ")("
                  << E.ev(x).c << ");\n";
                c++;
            }
            o << "RF_DEV void rf_emit(const RfParams& P, long long r, long long o)\n{\n" << body.str();
            for (auto& dcl : E.decls) o << "    " << dcl << "\n";
            o << w.str() << "}\n\n";
        }
        if (vectorize_ && !d.sp.filters.empty())
            throw LowerError("vectorised hash group-by with a filter: validity over groups is not lowered");
        o << "#define RF_MATERIALIZE 1\n#include \"rf_templates.cuh\"\n";
        o << "RF_MATERIALIZE_KERNELS(" << T << ", " << plan_.out_cols.size() << ")\n";
        plan_.kernels.clear();
        plan_.kernels.push_back({"rf_hg_init", 256, 0, KernelSpec::INIT});
        {
            const size_t head = ((size_t)kHotSlotsPerKey * HK * 9 + 15) / 16 * 16;
            const size_t smem = head + ((size_t)HW * HK + (size_t)HW * 32) * LL * 8 + (size_t)(HK + 15) / 16 * 16;
            plan_.kernels.push_back({"rf_hg_agg", HT, smem, KernelSpec::MAIN});
        }
        plan_.kernels.push_back({"rf_count", T, 0, KernelSpec::COUNT});
        plan_.kernels.push_back({"rf_scan", 1024, 0, KernelSpec::SCAN});
        plan_.kernels.push_back({"rf_scatter", T, 0, KernelSpec::SCATTER});
        plan_.aggs = L;
        plan_.device_range = false;
        std::fill(plan_.needs_index.begin(), plan_.needs_index.end(), 0);
        plan_.source = o.str();
        if (d.sp.iter->type.btype != INT64) throw LowerError("hash group-by keys must be int64");
    }

    // Merge co-iteration (InterSpace, iter_space.cpp:217-250,318-364): the loop walks the
    // sorted iterator columns of every vector and emits a row where all of them hold the same
    // value.  Here each row r of the first vector is an element: its partner in vector k is found
    // by binary search - the row at (first row of the key in k) + (rank of r among equal keys in
    // the first vector), which is how the two-pointer walk pairs duplicates.  Starts come from
    // Locate(max(lbs, first values)) as the merge's lower bound does; requires sorted columns.
    void lower_merge_join(const Op& op, const Drive& d)
    {
        plan_.kind = PlanKind::MERGE_JOIN;
        const Space& sp = d.sp;
        const int T = plan_.threads;
        if (sp.vecs.size() > 4) throw LowerError("merge co-iteration of more than 4 vectors");
        if (!(sp.iter->type.is_int() || sp.iter->type.is_idx())) throw LowerError("merge join over a non-integer iterator");
        std::string Ty = ctype(sp.iter->type);
        std::vector<int> slots;
        for (auto& v : sp.vecs) {
            slots.push_back(plan_.table_slot[v.first]);
            plan_.needs_index[v.first] = 1;
            if (fn_->inputs[v.first]->type.dim != 1) throw LowerError("merge join over a 2-d vector");
        }
        std::ostringstream o;
        o << "// generated by the reffine_gb300 lowering pass: " << fn_->name << " (merge co-iteration)\n";
        o << "#include \"rf_device.cuh\"\n\n";
        // range kernel: L, U, per-vector start rows
        {
            Emitter E(*this);
            bind_inputs(E);
            std::string first, last;
            for (size_t k = 0; k < slots.size(); k++) {
                std::string c = "P.t[" + std::to_string(slots[k]) + "].col[0]";
                std::string f = "rf_rd<" + Ty + ">(" + c + ", 0)";
                std::string l = "rf_rd<" + Ty + ">(" + c + ", " + c + ".len - 1)";
                first = first.empty() ? f : "rf_max<" + Ty + ">(" + f + ", " + first + ")";
                last = last.empty() ? l : "rf_min<" + Ty + ">(" + l + ", " + last + ")";
            }
            std::string L = bound_expr(E, sp.lbs, first, true, sp.iter->type);
            std::string U = sp.ubs.empty() ? last : bound_expr(E, sp.ubs, last, false, sp.iter->type);
            o << "extern \"C\" __global__ void rf_range(const __grid_constant__ RfParams P)\n{\n";
            o << "    if (threadIdx.x != 0 || blockIdx.x != 0) return;\n";
            for (auto& dcl : E.decls) o << "    " << dcl << "\n";
            o << "    const " << Ty << " L = " << L << ";\n    const " << Ty << " U = " << U << ";\n";
            o << "    bool empty = false;\n";
            for (size_t k = 0; k < slots.size(); k++) {
                std::string t = "P.t[" + std::to_string(slots[k]) + "]";
                o << "    long long s" << k << " = " << t << ".col[0].len > 0 ? rf_locate(" << t << ".ix, (long long)L) : -1;\n";
                o << "    if (" << t << ".col[0].len == 0) empty = true; else if (s" << k << " < 0) { rf_set_err(P, RF_DEVERR_RANGE); empty = true; }\n";
            }
            o << "    P.range[0] = empty ? 0 : s0;\n    P.range[1] = empty ? 0 : P.t[" << slots[0] << "].col[0].len;\n";
            o << "    P.range[2] = (long long)L;\n    P.range[3] = (long long)U;\n";
            for (size_t k = 1; k < slots.size(); k++) o << "    P.range[" << 3 + k << "] = s" << k << " < 0 ? 0 : s" << k << ";\n";
            o << "}\n\n";
            plan_.kernels.push_back({"rf_range", 32, 0, KernelSpec::RANGE});
            plan_.device_range = true;
        }
        o << "RF_DEV long long rf_lower_bound(const RfCol& c, long long lo, long long hi, " << Ty << " key)\n{\n";
        o << "    while (lo < hi) { long long mid = (lo + hi) >> 1; if (rf_ld<" << Ty << ">(c.data, mid) < key) lo = mid + 1; else hi = mid; }\n";
        o << "    return lo;\n}\n\n";
        auto body_of = [&](Emitter& E, std::ostringstream& b) -> std::string {
            std::string a = "P.t[" + std::to_string(slots[0]) + "].col[0]";
            b << "    const " << Ty << " it = rf_ld<" << Ty << ">(" << a << ".data, r);\n";
            b << "    const long long rank = r - rf_lower_bound(" << a << ", P.range[0], r, it);\n";
            b << "    bool mt = rf_valid(" << a << ".valid, r) && it >= (" << Ty << ")P.range[2] && it <= (" << Ty << ")P.range[3];\n";
            E.vec_iter_idx[{sp.vecs[0].second.get(), sp.iter.get()}] = "r";
            for (size_t k = 1; k < slots.size(); k++) {
                std::string c = "P.t[" + std::to_string(slots[k]) + "].col[0]";
                std::string j = "j" + std::to_string(k);
                b << "    const long long " << j << " = rf_lower_bound(" << c << ", P.range[" << 3 + k << "], " << c
                  << ".len, it) + rank;\n";
                b << "    mt = mt && " << j << " < " << c << ".len && rf_ld<" << Ty << ">(" << c << ".data, " << j
                  << ") == it && rf_valid(" << c << ".valid, " << j << ");\n";
                E.vec_iter_idx[{sp.vecs[k].second.get(), sp.iter.get()}] = j;
            }
            E.bind(op.iters[0], E.scalar("it", sp.iter->type));
            std::string cond = "mt";
            for (auto& f : sp.filters) cond += " && (" + E.ev(f).c + ")";
            return cond;
        };
        {
            Emitter E(*this);
            bind_inputs(E);
            std::ostringstream b;
            std::string cond = body_of(E, b);
            o << "RF_DEV bool rf_cond(const RfParams& P, long long r)\n{\n" << b.str();
            for (auto& dcl : E.decls) o << "    " << dcl << "\n";
            o << "    return " << cond << ";\n}\n\n";
        }
        {
            Emitter E(*this);
            bind_inputs(E);
            E.in_bounds_rows = false;
            std::ostringstream b;
            body_of(E, b);
            std::ostringstream w;
            size_t c = 0;
            w << "    ((" << Ty << "*)((void* const*)P.aux0)[" << c++ << "])[o] = it;\n";
            for (auto& x : op.outputs) {
                w << "    ((" << ctype(x->type) << "*)((void* const*)P.aux0)[" << c << "])[o] = (" << ctype(x->type) << ")("
                  << E.ev(x).c << ");\n";
                c++;
            }
            o << "RF_DEV void rf_emit(const RfParams& P, long long r, long long o)\n{\n" << b.str();
            for (auto& dcl : E.decls) o << "    " << dcl << "\n";
            o << w.str() << "}\n\n";
        }
        o << "#define RF_MATERIALIZE 1\n#include \"rf_templates.cuh\"\n";
        o << "RF_MATERIALIZE_KERNELS(" << T << ", " << plan_.out_cols.size() << ")\n";
        if (vectorize_) {
            plan_.kernels.push_back({"rf_write_all", T, 0, KernelSpec::FINAL});
        } else {
            plan_.kernels.push_back({"rf_count", T, 0, KernelSpec::COUNT});
            plan_.kernels.push_back({"rf_scan", 1024, 0, KernelSpec::SCAN});
            plan_.kernels.push_back({"rf_scatter", T, 0, KernelSpec::SCATTER});
        }
        plan_.source = o.str();
    }

    // Op over the union of two vectors (UnionSpace, iter_space.cpp:278-316, walked as JointSpace,
    // :217-250): Op([t], In(t, A) | In(t, B), outputs) over two 1-d vectors with sorted iterator
    // columns.  The walk visits the merged key sequence: at each step t is the smaller of the two
    // current keys, the side(s) holding t advance, and Element(A, t) / Element(B, t) read each
    // side's current row (the row holding t, or the lagging side's next row).  Both sides start
    // at row 0 and a side past its end takes no further part (its reads give 0).
    // A key v held cA times in A and cB times in B takes max(cA, cB) visits; visit j of v pairs
    // A row lA(v) + j with B row lB(v) + j while both exist.  Its position in the walk is
    //     lA(v) + lB(v) - M(lA(v)) + j,
    // lX(v) the first row of X with key >= v and M(i) the number of paired A rows before row i.
    // Kernels: rf_u_flags marks each paired A row, an exclusive scan gives M, rf_u_total the
    // number of visits, and rf_u_emit lets every A row and every unpaired B row write its visit
    // at its position - no compaction pass.  iter_cond (a side alive with a valid iterator) is
    // the validity bit of a vectorised output; without vectorize every visit is a row (inputs
    // whose iterator columns hold nulls are refused at run time then).
    void lower_union_op(const Op& op, const Expr& left, const Expr& right)
    {
        plan_.kind = PlanKind::UNION_MERGE;
        const int T = plan_.threads;
        if (op.iters.size() != 1) throw LowerError("union over several iterators");
        const Expr& it = op.iters[0];
        if (!(it->type == types::INT64_T || it->type.is_idx())) throw LowerError("union over a non-int64 iterator");
        int in[2];
        Expr vec[2];
        const Expr sides[2] = {resolve(left), resolve(right)};
        for (int k = 0; k < 2; k++) {
            if (sides[k]->kind != NodeKind::IN) throw LowerError("a union of iteration spaces other than two vectors");
            auto i = as<In>(sides[k]);
            if (i->iter.get() != it.get()) throw LowerError("union over another iterator");
            vec[k] = resolve(i->vec);
            auto f = input_index_.find(vec[k].get());
            if (f == input_index_.end()) throw LowerError("union over a non-input vector");
            in[k] = f->second;
            const DataType& vt = fn_->inputs[in[k]]->type;
            if (vt.dim != 1) throw LowerError("union over a 2-d vector");
            if (!(vt.dtypes[0] == types::INT64_T || vt.dtypes[0].is_idx())) throw LowerError("union over non-int64 keys");
            note_col(in[k], 0);
        }
        if (in[0] == in[1]) throw LowerError("union of a vector with itself");
        // no driving table: the walk's domain is both vectors' rows (nA + nB), not one table's
        plan_.drive_input = -1;
        {
            HostExpr lo, a, b, sum;
            lo.kind = HostExpr::CONST;
            lo.value = 0;
            a.kind = b.kind = HostExpr::LEN;
            a.input = in[0];
            b.input = in[1];
            a.col = b.col = 0;
            sum.kind = HostExpr::ADD;
            sum.args = {a, b};
            plan_.row_lo = lo;
            plan_.row_hi = sum;
        }
        plan_.device_range = false;
        plan_.union_inputs[0] = in[0];
        plan_.union_inputs[1] = in[1];
        const std::string A = "P.t[" + std::to_string(plan_.table_slot[in[0]]) + "].col[0]";
        const std::string B = "P.t[" + std::to_string(plan_.table_slot[in[1]]) + "].col[0]";
        std::ostringstream o;
        o << "// generated by the reffine_gb300 lowering pass: " << fn_->name << " (union merge co-iteration)\n";
        o << "#include \"rf_device.cuh\"\n\n";
        o << "// first row of sorted int64 column c (n rows) whose key is >= key (> key when upper)\n";
        o << "RF_DEV long long rf_u_bound(const RfCol& c, long long n, long long key, bool upper)\n{\n";
        o << "    long long lo = 0, hi = n;\n    const long long* k = (const long long*)c.data;\n";
        o << "    while (lo < hi) {\n        const long long m = (lo + hi) >> 1;\n        const long long x = __ldg(k + m);\n";
        o << "        if (x < key || (upper && x == key)) lo = m + 1; else hi = m;\n    }\n    return lo;\n}\n\n";
        o << "extern \"C\" __global__ void __launch_bounds__(256) rf_u_flags(const __grid_constant__ RfParams P)\n{\n";
        o << "    long long* M = (long long*)P.aux4;\n    const long long nA = " << A << ".len, nB = " << B << ".len;\n";
        o << "    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nA; i += (long long)gridDim.x * blockDim.x) {\n";
        o << "        const long long v = rf_ld<int64_t>(" << A << ".data, i);\n";
        o << "        const long long a = i - rf_u_bound(" << A << ", nA, v, false);\n";
        o << "        const long long lB = rf_u_bound(" << B << ", nB, v, false), cB = rf_u_bound(" << B << ", nB, v, true) - lB;\n";
        o << "        M[i] = a < cB ? 1 : 0;\n    }\n";
        o << "    if (blockIdx.x == 0 && threadIdx.x == 0) M[nA] = 0;\n}\n\n";
        o << "extern \"C\" __global__ void rf_u_total(const __grid_constant__ RfParams P)\n{\n";
        o << "    if (threadIdx.x != 0 || blockIdx.x != 0) return;\n";
        o << "    const long long nA = " << A << ".len, nB = " << B << ".len;\n";
        o << "    ((long long*)P.aux3)[0] = nA + nB - ((const long long*)P.aux4)[nA];\n}\n\n";
        // the visit's outputs
        Emitter E(*this);
        bind_inputs(E);
        E.in_bounds_rows = false;
        E.vec_iter_idx[{vec[0].get(), it.get()}] = "li";
        E.vec_iter_idx[{vec[1].get(), it.get()}] = "ri";
        E.bind(op.iters[0], E.scalar("it", it->type));
        std::ostringstream w;
        size_t c = 0;
        w << "    ((" << ctype(it->type) << "*)((void* const*)P.aux0)[" << c++ << "])[o] = it;\n";
        for (auto& x : op.outputs) {
            w << "    ((" << ctype(x->type) << "*)((void* const*)P.aux0)[" << c << "])[o] = (" << ctype(x->type) << ")("
              << E.ev(x).c << ");\n";
            c++;
        }
        o << "RF_DEV void rf_u_write(const RfParams& P, long long li, long long ri, long long v, long long o)\n{\n";
        o << "    const " << ctype(it->type) << " it = (" << ctype(it->type) << ")v;\n";
        for (auto& dcl : E.decls) o << "    " << dcl << "\n";
        o << w.str() << "}\n\n";
        o << "extern \"C\" __global__ void __launch_bounds__(" << T << ") rf_u_emit(const __grid_constant__ RfParams P)\n{\n";
        o << "    const long long* M = (const long long*)P.aux4;\n    const long long nA = " << A << ".len, nB = " << B
          << ".len;\n    const long long V = ((const long long*)P.aux3)[0];\n    long long nulls = 0;\n";
        o << "    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < nA + nB; r += (long long)gridDim.x * blockDim.x) {\n";
        o << "        long long v, li, ri, pos;\n";
        o << "        if (r < nA) {\n            li = r;\n            v = rf_ld<int64_t>(" << A << ".data, li);\n";
        o << "            const long long lA = rf_u_bound(" << A << ", nA, v, false), a = li - lA;\n";
        o << "            const long long lB = rf_u_bound(" << B << ", nB, v, false), cB = rf_u_bound(" << B << ", nB, v, true) - lB;\n";
        o << "            ri = a < cB ? lB + a : lB + cB;\n            pos = lA + lB - M[lA] + a;\n";
        o << "        } else {\n            ri = r - nA;\n            v = rf_ld<int64_t>(" << B << ".data, ri);\n";
        o << "            const long long lB = rf_u_bound(" << B << ", nB, v, false), b = ri - lB;\n";
        o << "            const long long lA = rf_u_bound(" << A << ", nA, v, false), cA = rf_u_bound(" << A << ", nA, v, true) - lA;\n";
        o << "            if (b < cA) continue;  // paired with A row lA + b, which writes the visit\n";
        o << "            li = lA + cA;\n            pos = lA + lB - M[lA] + b;\n        }\n";
        // keys out of order (the walk needs sorted iterator columns) can only move a visit, never
        // past the output: positions are checked against the visit count
        o << "        if (pos < 0 || pos >= V) { rf_set_err(P, RF_DEVERR_RANGE); continue; }\n";
        o << "        rf_u_write(P, li, ri, v, pos);\n";
        if (vectorize_) {
            o << "        const bool ok = (li < nA && rf_valid(" << A << ".valid, li)) || (ri < nB && rf_valid(" << B
              << ".valid, ri));\n";
            o << "        if (ok)\n            for (int col = 0; col < " << plan_.out_cols.size()
              << "; col++) atomicOr(((unsigned**)P.aux1)[col] + (pos >> 5), 1u << (pos & 31));\n";
            o << "        else\n            nulls++;\n";
        }
        o << "    }\n";
        o << "    if (nulls) atomicAdd((unsigned long long*)P.aux3 + 1, (unsigned long long)nulls);\n}\n";
        plan_.kernels.clear();
        plan_.kernels.push_back({"rf_u_flags", 256, 0, KernelSpec::SEGCOUNT});
        plan_.kernels.push_back({"", 0, 0, KernelSpec::SEGSCAN});
        plan_.kernels.push_back({"rf_u_total", 32, 0, KernelSpec::RANGE});
        plan_.kernels.push_back({"rf_u_emit", T, 0, KernelSpec::SCATTER});
        plan_.source = o.str();
    }

    // Op over several iterators (NestedSpace, iter_space.cpp:366-452): the loop nest visits the
    // outer iterator's range and, for each of its values, the inner ones in order.  Lowered here
    // for rectangular nests: every iterator ranges over bounds of constants and scalar inputs
    // (no vector, no bound that names another iterator).  The nest's visits are numbered in loop
    // order and each number is decomposed into the iterators' values.  As in the reference's
    // loop, an inner level that runs past its upper bound is visited once more (iter_cond false,
    // a null row of the vectorised output) before the next outer value resets it: a level j > 0
    // with n_j values takes S_j = n_j * S_{j+1} + 1 visits (S_k = 1 past the innermost), the
    // outermost n_0 * S_1.  The non-vectorised output keeps the valid visits, in order.
    void lower_nested_op(const Op& op)
    {
        plan_.kind = PlanKind::MATERIALIZE;
        const int T = plan_.threads;
        const size_t K = op.iters.size();
        std::set<const ExprNode*> vars;
        for (auto& s : fn_->inputs)
            if (s->type.is_val()) vars.insert(s.get());
        std::vector<Space> sps(K);
        for (size_t j = 0; j < K; j++) {
            Space& sp = sps[j];
            sp.iter = op.iters[j];
            if (!(sp.iter->type.is_int() || sp.iter->type.is_idx())) throw LowerError("nested Op over a non-integer iterator");
            space_of(op.pred, sp.iter, vars, sp);
            if (sp.has_vec) throw LowerError("nested Op over a vector is not lowered");
            if (sp.lbs.empty() || sp.ubs.empty()) throw LowerError("unbounded iteration space in a nested Op");
            for (auto* bs : {&sp.lbs, &sp.ubs})
                for (auto& b : *bs)
                    for (auto& it : op.iters)
                        if (mentions(b, it.get(), fn_->tbl)) throw LowerError("nested Op bound over another iterator");
            for (auto& f : sp.filters)
                for (auto& it : op.iters)
                    if (it.get() != sp.iter.get() && mentions(f, it.get(), fn_->tbl))
                        throw LowerError("nested Op filter over another iterator");
        }
        // host-side visit count: n_j = max(U_j - L_j + 1, 0)
        auto n_host = [&](const Space& sp) {
            HostExpr one, zero, up, d, n;
            one.kind = HostExpr::CONST;
            one.value = 1;
            zero.kind = HostExpr::CONST;
            zero.value = 0;
            up.kind = HostExpr::ADD;
            up.args = {minmax_host(sp.ubs, false), one};
            d.kind = HostExpr::SUB;
            d.args = {up, minmax_host(sp.lbs, true)};
            n.kind = HostExpr::MAX;
            n.args = {d, zero};
            return n;
        };
        HostExpr S;
        S.kind = HostExpr::CONST;
        S.value = 1;
        for (size_t j = K; j-- > 0;) {
            HostExpr m;
            m.kind = HostExpr::MUL;
            m.args = {n_host(sps[j]), S};
            if (j > 0) {
                HostExpr one, a;
                one.kind = HostExpr::CONST;
                one.value = 1;
                a.kind = HostExpr::ADD;
                a.args = {m, one};
                S = a;
            } else {
                S = m;
            }
        }
        HostExpr lo;
        lo.kind = HostExpr::CONST;
        lo.value = 0;
        plan_.row_lo = lo;
        plan_.row_hi = S;
        plan_.device_range = false;
        std::ostringstream src;
        src << "// generated by the reffine_gb300 lowering pass: " << fn_->name << " (nested Op)\n";
        src << "#include \"rf_device.cuh\"\n\n";
        // decomposition of visit r into the iterators it0..it{K-1} and its validity
        auto bind_nest = [&](Emitter& E, std::ostringstream& b) -> std::string {
            bind_inputs(E);
            for (size_t j = 0; j < K; j++) {
                std::string Tj = ctype(sps[j].iter->type), J = std::to_string(j);
                b << "    const long long L" << J << " = (long long)(" << bound_expr(E, sps[j].lbs, "", true, sps[j].iter->type)
                  << ");\n";
                b << "    long long n" << J << " = (long long)(" << bound_expr(E, sps[j].ubs, "", false, sps[j].iter->type)
                  << ") - L" << J << " + 1;\n    if (n" << J << " < 0) n" << J << " = 0;\n";
            }
            // S_j: visits of level j's block (S_K = 1)
            b << "    long long S" << K << " = 1;\n";
            for (size_t j = K; j-- > 1;)
                b << "    const long long S" << j << " = n" << j << " * S" << j + 1 << " + 1;\n";
            b << "    bool ok = true;\n    long long p = r;\n";
            for (size_t j = 0; j < K; j++) {
                std::string J = std::to_string(j), J1 = std::to_string(j + 1);
                b << "    long long i" << J << ";\n";
                if (j == 0) {
                    b << "    i0 = L0 + p / S1;\n    p = p % S1;\n";
                } else {
                    b << "    if (!ok) { i" << J << " = L" << J << "; }\n";
                    b << "    else if (p == n" << J << " * S" << J1 << ") { i" << J << " = L" << J << " + n" << J
                      << "; ok = false; }\n";
                    b << "    else { i" << J << " = L" << J << " + p / S" << J1 << "; p = p % S" << J1 << "; }\n";
                }
                b << "    const " << ctype(sps[j].iter->type) << " it" << J << " = (" << ctype(sps[j].iter->type) << ")i"
                  << J << ";\n";
                E.bind(op.iters[j], E.scalar("it" + J, sps[j].iter->type));
            }
            b << "    (void)p;\n";
            std::string cond = "ok";
            for (auto& sp : sps)
                for (auto& f : sp.filters) cond += " && (" + E.ev(f).c + ")";
            return cond;
        };
        {
            Emitter E(*this);
            std::ostringstream b;
            std::string cond = bind_nest(E, b);
            src << "RF_DEV bool rf_cond(const RfParams& P, long long r)\n{\n" << b.str();
            for (auto& dcl : E.decls) src << "    " << dcl << "\n";
            src << "    return " << cond << ";\n}\n\n";
        }
        {
            Emitter E(*this);
            std::ostringstream b;
            bind_nest(E, b);
            std::ostringstream w;
            size_t c = 0;
            for (auto& i : op.iters) {
                w << "    ((" << ctype(i->type) << "*)((void* const*)P.aux0)[" << c << "])[o] = (" << ctype(i->type)
                  << ")(" << E.ev(i).c << ");\n";
                c++;
            }
            for (auto& x : op.outputs) {
                w << "    ((" << ctype(x->type) << "*)((void* const*)P.aux0)[" << c << "])[o] = (" << ctype(x->type)
                  << ")(" << E.ev(x).c << ");\n";
                c++;
            }
            src << "RF_DEV void rf_emit(const RfParams& P, long long r, long long o)\n{\n" << b.str();
            for (auto& dcl : E.decls) src << "    " << dcl << "\n";
            src << w.str() << "}\n\n";
        }
        src << "#define RF_MATERIALIZE 1\n#include \"rf_templates.cuh\"\n";
        src << "RF_MATERIALIZE_KERNELS(" << T << ", " << plan_.out_cols.size() << ")\n";
        if (vectorize_) {
            plan_.kernels.push_back({"rf_write_all", T, 0, KernelSpec::FINAL});
        } else {
            plan_.kernels.push_back({"rf_count", T, 0, KernelSpec::COUNT});
            plan_.kernels.push_back({"rf_scan", 1024, 0, KernelSpec::SCAN});
            plan_.kernels.push_back({"rf_scatter", T, 0, KernelSpec::SCATTER});
        }
        plan_.source = src.str();
    }

    void lower_op(const Expr& opx)
    {
        const Op& op = *as<Op>(opx);
        plan_.out_is_table = true;
        plan_.out_dim = (int)op.iters.size();
        for (auto& i : op.iters) plan_.out_cols.push_back(i->type);
        for (auto& o : op.outputs) {
            if (!o->type.is_primitive()) throw LowerError("data type not supported " + o->type.str(), false);
            plan_.out_cols.push_back(o->type);
        }
        if ((int)plan_.out_cols.size() > RF_MAX_COLS_) throw LowerError("too many output columns");
        if (op.iters.size() > 1) {
            lower_nested_op(op);
            return;
        }
        {
            Expr pred = resolve(op.pred);
            if (is_nary(pred, MathOp::OR)) {
                lower_union_op(op, as<NaryExpr>(pred)->args[0], as<NaryExpr>(pred)->args[1]);
                return;
            }
        }
        Drive d;
        d.sp = op_space(op);
        drive_rows(d);
        if (d.sp.n_vecs > 1) {
            lower_merge_join(op, d);
            return;
        }
        plan_.kind = PlanKind::MATERIALIZE;
        const int T = plan_.threads;
        std::ostringstream src;
        src << "// generated by the reffine_gb300 lowering pass: " << fn_->name << " (Op materialisation)\n";
        src << "#include \"rf_device.cuh\"\n\n";
        emit_range_kernels(src, d);

        // an Op over a 2-d vector whose outputs reduce each element's sub-vector
        // (LoopGen::visit(Element) dim 2 -> SubVector of run ends, loopgen.cpp:34-38)
        const Reduce* seg = nullptr;
        std::vector<Leaf> seg_leaves;
        std::vector<int> seg_act;
        if (d.sp.has_vec && fn_->inputs[d.input]->type.dim == 2) {
            std::vector<const Reduce*> reds;
            for (auto& o : op.outputs) find_reduces(o, reds);
            for (auto& f : d.sp.filters) find_reduces(f, reds);
            std::sort(reds.begin(), reds.end());
            reds.erase(std::unique(reds.begin(), reds.end()), reds.end());
            if (reds.size() > 1) throw LowerError("more than one nested Reduce per element");
            if (reds.size() == 1) {
                seg = reds[0];
                if (seg->vec->kind != NodeKind::ELEMENT) throw LowerError("nested Reduce over a non-element vector");
                auto el = as<Element>(seg->vec);
                if (resolve(el->vec).get() != resolve(d.sp.vec_node).get() || el->iter.get() != op.iters[0].get())
                    throw LowerError("nested Reduce over another vector's element");
                const DataType& vt = fn_->inputs[d.input]->type;
                if (vt.encodings[0] != RUNEND) {
                    lower_hash_group(op, d, *seg);
                    return;
                }
                plan_.kind = PlanKind::SEG_REDUCE;
                collect_leaves(*seg, seg->type, {}, seg_leaves);
                for (size_t i = 0; i < seg_leaves.size(); i++)
                    if (seg_leaves[i].op != AggOp::NONE) seg_act.push_back((int)i);
                emit_acc(src, seg_leaves, seg_act);
                plan_.acc_bytes = std::max<size_t>(8, seg_act.size() * 8);
                Drive rd;
                rd.subvec = true;
                rd.input = d.input;
                rd.slot = d.slot;
                emit_row(src, *seg, rd, seg_leaves, seg_act);
                emit_seg_kernels(src, d);
            }
        }
        auto bind_seg = [&](Emitter& E, std::ostringstream& body) {
            if (!seg) return;
            body << "    RfAcc SA;\n    rf_fold(P, r, SA);\n";
            Val st = seg_state(E, body, *seg, seg_leaves);
            E.node_bind[(const ExprNode*)seg] = st;
        };
        {
            Emitter E(*this);
            bind_inputs(E);
            std::ostringstream body;
            std::string cond = bind_op_row(E, op, d, body);
            bool needs = false;
            for (auto& f : d.sp.filters) {
                std::vector<const Reduce*> rr;
                find_reduces(f, rr);
                needs |= !rr.empty();
            }
            if (needs) bind_seg(E, body);
            src << "RF_DEV bool rf_cond(const RfParams& P, long long r)\n{\n" << body.str();
            for (auto& dcl : E.decls) src << "    " << dcl << "\n";
            src << "    return " << cond << ";\n}\n\n";
        }
        {
            Emitter E(*this);
            bind_inputs(E);
            std::ostringstream body;
            bind_op_row(E, op, d, body);
            bind_seg(E, body);
            std::ostringstream w;
            size_t c = 0;
            for (auto& i : op.iters) {
                w << "    ((" << ctype(i->type) << "*)((void* const*)P.aux0)[" << c << "])[o] = (" << ctype(i->type)
                  << ")(" << E.ev(i).c << ");\n";
                c++;
            }
            for (auto& o : op.outputs) {
                w << "    ((" << ctype(o->type) << "*)((void* const*)P.aux0)[" << c << "])[o] = (" << ctype(o->type)
                  << ")(" << E.ev(o).c << ");\n";
                c++;
            }
            src << "RF_DEV void rf_emit(const RfParams& P, long long r, long long o)\n{\n" << body.str();
            for (auto& dcl : E.decls) src << "    " << dcl << "\n";
            src << w.str() << "}\n\n";
        }
        src << "#define RF_MATERIALIZE 1\n#include \"rf_templates.cuh\"\n";
        src << "RF_MATERIALIZE_KERNELS(" << T << ", " << plan_.out_cols.size() << ")\n";
        if (vectorize_) {
            plan_.kernels.push_back({"rf_write_all", T, 0, KernelSpec::FINAL});
        } else {
            plan_.kernels.push_back({"rf_count", T, 0, KernelSpec::COUNT});
            plan_.kernels.push_back({"rf_scan", 1024, 0, KernelSpec::SCAN});
            plan_.kernels.push_back({"rf_scatter", T, 0, KernelSpec::SCATTER});
        }
        plan_.source = src.str();
    }

    std::shared_ptr<Func> fn_;
    bool vectorize_;
    int threads_;
    Plan plan_;
    std::map<const ExprNode*, int> input_index_;
};

}  // namespace

size_t c_align(const DataType& t)
{
    if (t.is_struct()) {
        size_t a = 1;
        for (auto& d : t.dtypes) a = std::max(a, c_align(d));
        return a;
    }
    return t.size();
}

size_t c_size(const DataType& t)
{
    if (t.is_struct()) {
        size_t off = 0;
        for (auto& d : t.dtypes) {
            size_t al = c_align(d);
            off = (off + al - 1) / al * al + c_size(d);
        }
        size_t al = c_align(t);
        return (off + al - 1) / al * al;
    }
    return t.size();
}

Plan lower(const std::shared_ptr<Func>& fn, bool vectorize, int threads)
{
    if (threads != 128 && threads != 256 && threads != 512) throw LowerError("block size must be 128, 256 or 512");
    return Lowerer(fn, vectorize, threads).run();
}

}  // namespace rfg
