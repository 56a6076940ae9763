// Reffine IR for the GB300 backend: types, nodes, builder DSL, text form.
//
// The node set, the typing rules and the builder names follow Reffine's own IR so that query
// code written against Reffine compiles against this header unchanged:
//   types     include/reffine/base/type.h:17-250   (BaseType, EncodeType, DataType, valty/iterty/rowty)
//   nodes     include/reffine/ir/expr.h, op.h, op_to_loop.h, stmt.h (Const, NaryExpr, Select, Cast,
//             Get, New, Op, Element, In, Reduce, SubVector, Length, Locate, ReadData, Func)
//   DSL       include/reffine/builder/reffiner.h:34-187 (_expr<T> operators, _op/_red/_in/_sym/...)
// What differs: the loop-level IR (Loop/Alloc/Load/Store, loop.h) is not part of this header;
// the GPU backend lowers the functional IR directly.  Every Func prints to an S-expression text
// (Printer) and parses back (Parser); that text is the query description the C-ABI takes
// (rf_plan_compile in include/rf_gpu.h).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

namespace reffine {

using std::make_shared;
using std::shared_ptr;
using std::string;
using std::vector;

enum BaseType {
    UNKNOWN = -1, VOID, BOOL, INT8, INT16, INT32, INT64, UINT8, UINT16, UINT32, UINT64,
    FLOAT32, FLOAT64, STRUCT, PTR, STR, IDX, VECTOR,
};

enum EncodeType { FLAT, RUNEND };

struct DataType {
    BaseType btype;
    vector<DataType> dtypes;
    size_t dim;
    vector<EncodeType> encodings;

    explicit DataType(BaseType b = VOID, vector<DataType> d = {}, size_t dm = 0, vector<EncodeType> e = {})
        : btype(b), dtypes(std::move(d)), dim(dm), encodings(std::move(e))
    {
        if (btype == VECTOR && encodings.empty()) encodings.assign(dtypes.size(), FLAT);
        if (btype == STRUCT && dtypes.empty()) throw std::runtime_error("empty struct type");
        if (btype == VECTOR && (dim == 0 || dtypes.size() < dim || encodings.size() != dtypes.size()))
            throw std::runtime_error("malformed vector type");
    }
    // equality ignores encodings, as type.h:71-75 does
    bool operator==(const DataType& o) const { return btype == o.btype && dtypes == o.dtypes && dim == o.dim; }
    bool operator!=(const DataType& o) const { return !(*this == o); }
    bool operator<(const DataType& o) const { return str() < o.str(); }

    bool is_struct() const { return btype == STRUCT; }
    bool is_vector() const { return btype == VECTOR; }
    bool is_idx() const { return btype == IDX; }
    bool is_void() const { return btype == VOID; }
    bool is_val() const { return !is_vector(); }
    bool is_float() const { return btype == FLOAT32 || btype == FLOAT64; }
    bool is_int() const { return btype >= INT8 && btype <= UINT64; }
    bool is_unsigned() const { return btype >= UINT8 && btype <= UINT64; }
    bool is_signed() const { return (btype >= INT8 && btype <= INT64) || is_float(); }
    bool is_primitive() const { return is_int() || is_float() || is_idx() || btype == BOOL; }

    DataType valty() const
    {
        if (!is_vector()) throw std::runtime_error("valty of non-vector");
        vector<DataType> d(dtypes.begin() + 1, dtypes.end());
        vector<EncodeType> e(encodings.begin() + 1, encodings.end());
        if (dim == 1) return DataType(STRUCT, d);
        return DataType(VECTOR, d, dim - 1, e);
    }
    DataType iterty() const
    {
        if (!is_vector()) throw std::runtime_error("iterty of non-vector");
        return dtypes[0];
    }
    DataType rowty() const
    {
        if (!is_vector()) throw std::runtime_error("rowty of non-vector");
        return DataType(STRUCT, dtypes);
    }
    size_t size() const
    {
        switch (btype) {
            case BOOL: case INT8: case UINT8: return 1;
            case INT16: case UINT16: return 2;
            case INT32: case UINT32: case FLOAT32: return 4;
            case INT64: case UINT64: case FLOAT64: case IDX: case PTR: return 8;
            default: throw std::runtime_error("size of non-primitive type");
        }
    }
    // C/C++ type name, as type.h:206-240 (cppstr)
    string cppstr() const
    {
        switch (btype) {
            case VOID: return "void";
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
            case VECTOR: return "ArrowTable*";
            default: throw std::runtime_error("no C type for " + str());
        }
    }
    // short name, used in the text form
    string str() const
    {
        switch (btype) {
            case VOID: return "void";
            case BOOL: return "bool";
            case INT8: return "i8";
            case UINT8: return "u8";
            case INT16: return "i16";
            case UINT16: return "u16";
            case INT32: return "i32";
            case UINT32: return "u32";
            case INT64: return "i64";
            case UINT64: return "u64";
            case FLOAT32: return "f32";
            case FLOAT64: return "f64";
            case IDX: return "idx";
            case STRUCT: {
                string s = "(struct";
                for (auto& d : dtypes) s += " " + d.str();
                return s + ")";
            }
            case VECTOR: {
                string s = "(vector " + std::to_string(dim) + " (";
                for (size_t i = 0; i < dtypes.size(); i++) s += (i ? " " : "") + dtypes[i].str();
                s += ") (";
                for (size_t i = 0; i < encodings.size(); i++)
                    s += string(i ? " " : "") + (encodings[i] == RUNEND ? "runend" : "flat");
                return s + "))";
            }
            default: throw std::runtime_error("invalid type");
        }
    }
};

namespace types {
static const DataType VOID_T(VOID);
static const DataType BOOL_T(BOOL);
static const DataType INT8_T(INT8);
static const DataType INT16_T(INT16);
static const DataType INT32_T(INT32);
static const DataType INT64_T(INT64);
static const DataType UINT8_T(UINT8);
static const DataType UINT16_T(UINT16);
static const DataType UINT32_T(UINT32);
static const DataType UINT64_T(UINT64);
static const DataType FLOAT32_T(FLOAT32);
static const DataType FLOAT64_T(FLOAT64);
static const DataType IDX_T(IDX);
template <typename H> struct Converter { static const BaseType btype = UNKNOWN; };
template <> struct Converter<bool> { static const BaseType btype = BOOL; };
template <> struct Converter<char> { static const BaseType btype = INT8; };
template <> struct Converter<int8_t> { static const BaseType btype = INT8; };
template <> struct Converter<int16_t> { static const BaseType btype = INT16; };
template <> struct Converter<int32_t> { static const BaseType btype = INT32; };
template <> struct Converter<int64_t> { static const BaseType btype = INT64; };
template <> struct Converter<uint8_t> { static const BaseType btype = UINT8; };
template <> struct Converter<uint16_t> { static const BaseType btype = UINT16; };
template <> struct Converter<uint32_t> { static const BaseType btype = UINT32; };
template <> struct Converter<uint64_t> { static const BaseType btype = UINT64; };
template <> struct Converter<float> { static const BaseType btype = FLOAT32; };
template <> struct Converter<double> { static const BaseType btype = FLOAT64; };
// types::VEC<dim, Ts...> (type.h:383-392)
template <size_t dim, typename... Ts>
DataType VEC()
{
    return DataType(VECTOR, vector<DataType>{DataType(Converter<Ts>::btype)...}, dim);
}
template <typename... Ts>
DataType STRUCT()
{
    return DataType(BaseType::STRUCT, vector<DataType>{DataType(Converter<Ts>::btype)...});
}
}  // namespace types

enum class MathOp {
    ADD, SUB, MUL, DIV, MAX, MIN, MOD, SQRT, POW, ABS, NEG, CEIL, FLOOR,
    LT, LTE, GT, GTE, EQ, NOT, AND, OR, IMPLIES, IFF, FORALL, EXISTS,
};

inline const char* mathop_name(MathOp op)
{
    static const char* n[] = {"add", "sub", "mul", "div", "max", "min", "mod", "sqrt", "pow", "abs", "neg",
                              "ceil", "floor", "lt", "lte", "gt", "gte", "eq", "not", "and", "or",
                              "implies", "iff", "forall", "exists"};
    return n[(int)op];
}

enum class NodeKind {
    SYM, CONST, NARY, SELECT, CAST, GET, NEW, OP, ELEMENT, IN, REDUCE, SUBVECTOR, LENGTH, LOCATE, READDATA,
};

struct ExprNode {
    const DataType type;
    const NodeKind kind;
    ExprNode(DataType t, NodeKind k) : type(std::move(t)), kind(k) {}
    virtual ~ExprNode() {}
};
using Expr = shared_ptr<ExprNode>;

struct SymNode : ExprNode {
    const string name;
    SymNode(string n, DataType t) : ExprNode(std::move(t), NodeKind::SYM), name(std::move(n)) {}
    SymNode(string n, Expr e) : ExprNode(e->type, NodeKind::SYM), name(std::move(n)) {}
};
using Sym = shared_ptr<SymNode>;
using SymTable = std::map<Sym, Expr>;

// Const stores a double, as expr.h:76-85 does (int64 constants above 2^53 lose precision there too)
struct Const : ExprNode {
    const double val;
    Const(DataType t, double v) : ExprNode(std::move(t), NodeKind::CONST), val(v)
    {
        if (!type.is_primitive()) throw std::runtime_error("non-primitive constant");
    }
};

struct NaryExpr : ExprNode {
    MathOp op;
    vector<Expr> args;
    NaryExpr(DataType t, MathOp o, vector<Expr> a) : ExprNode(std::move(t), NodeKind::NARY), op(o), args(std::move(a))
    {
        if (args.empty() || args[0]->type.is_struct()) throw std::runtime_error("NaryExpr over a struct");
    }
    Expr arg(size_t i) const { return args[i]; }
    size_t size() const { return args.size(); }
};

struct Select : ExprNode {
    Expr cond, true_body, false_body;
    Select(Expr c, Expr t, Expr f)
        : ExprNode(t->type, NodeKind::SELECT), cond(std::move(c)), true_body(std::move(t)), false_body(std::move(f))
    {
        if (cond->type != types::BOOL_T) throw std::runtime_error("select condition is not bool");
        if (true_body->type != false_body->type) throw std::runtime_error("select branch types differ");
    }
};

struct Cast : ExprNode {
    Expr arg;
    Cast(DataType t, Expr a) : ExprNode(std::move(t), NodeKind::CAST), arg(std::move(a))
    {
        if (arg->type.is_struct() || type.is_struct()) throw std::runtime_error("cast of struct");
    }
};

struct Get : ExprNode {
    Expr val;
    size_t col;
    static DataType ty(const Expr& v, size_t c)
    {
        if (v->type.is_struct()) {
            if (c >= v->type.dtypes.size()) throw std::runtime_error("get: field out of range");
            return v->type.dtypes[c];
        }
        if (!v->type.is_primitive() || c != 0) throw std::runtime_error("get on non-struct");
        return v->type;
    }
    Get(Expr v, size_t c) : ExprNode(ty(v, c), NodeKind::GET), val(std::move(v)), col(c) {}
};

struct New : ExprNode {
    vector<Expr> vals;
    static DataType ty(const vector<Expr>& v)
    {
        vector<DataType> d;
        for (auto& e : v) d.push_back(e->type);
        return DataType(STRUCT, d);
    }
    explicit New(vector<Expr> v) : ExprNode(ty(v), NodeKind::NEW), vals(std::move(v)) {}
};

struct Op : ExprNode {
    vector<Sym> iters;
    Expr pred;
    vector<Expr> outputs;
    static DataType ty(const vector<Sym>& it, const vector<Expr>& out)
    {
        vector<DataType> d;
        for (auto& i : it) {
            if (!i->type.is_primitive()) throw std::runtime_error("op iterator must be primitive");
            d.push_back(i->type);
        }
        for (auto& o : out) {
            if (!o->type.is_val()) throw std::runtime_error("op output must be a value");
            d.push_back(o->type);
        }
        return DataType(VECTOR, d, it.size());
    }
    Op(vector<Sym> it, Expr p, vector<Expr> out)
        : ExprNode(ty(it, out), NodeKind::OP), iters(std::move(it)), pred(std::move(p)), outputs(std::move(out))
    {
    }
};

struct Element : ExprNode {
    Expr vec, iter;
    Element(Expr v, Expr i) : ExprNode(v->type.valty(), NodeKind::ELEMENT), vec(std::move(v)), iter(std::move(i))
    {
        if (iter->type != vec->type.iterty()) throw std::runtime_error("element: iterator type mismatch");
    }
};

struct In : ExprNode {
    Expr iter, vec;
    In(Expr i, Expr v) : ExprNode(types::BOOL_T, NodeKind::IN), iter(std::move(i)), vec(std::move(v))
    {
        if (iter->type != vec->type.iterty()) throw std::runtime_error("in: iterator type mismatch");
    }
};

using InitFnTy = std::function<Expr()>;
using AccFnTy = std::function<Expr(Expr, Expr)>;

// op.h:89-110.  The lambdas are applied once, to a fresh state symbol and a fresh value symbol
// (the value has the vector's row type), and the resulting expressions are kept.
struct Reduce : ExprNode {
    Expr vec;
    Expr init_expr;
    Sym state, val;
    Expr acc_expr;
    Reduce(Expr v, Expr init, Sym st, Sym vl, Expr acc)
        : ExprNode(init->type, NodeKind::REDUCE), vec(std::move(v)), init_expr(std::move(init)), state(std::move(st)),
          val(std::move(vl)), acc_expr(std::move(acc))
    {
        if (!vec->type.is_vector()) throw std::runtime_error("reduce over a non-vector");
        if (acc_expr->type != init_expr->type) throw std::runtime_error("reduce: acc and init types differ");
    }
    static shared_ptr<Reduce> make(Expr v, const InitFnTy& init, const AccFnTy& acc)
    {
        static int counter = 0;
        auto i = init();
        int k = counter++;
        auto st = make_shared<SymNode>("s" + std::to_string(k), i->type);
        auto vl = make_shared<SymNode>("v" + std::to_string(k), v->type.rowty());
        auto a = acc(st, vl);
        return make_shared<Reduce>(v, i, st, vl, a);
    }
};

struct SubVector : ExprNode {
    Expr vec, start, end;
    SubVector(Expr v, Expr s, Expr e)
        : ExprNode(v->type.valty(), NodeKind::SUBVECTOR), vec(std::move(v)), start(std::move(s)), end(std::move(e))
    {
        if (!start->type.is_idx() || !end->type.is_idx()) throw std::runtime_error("subvector bounds must be idx");
    }
};

struct Length : ExprNode {
    Expr vec;
    size_t col;
    Length(Expr v, size_t c) : ExprNode(types::IDX_T, NodeKind::LENGTH), vec(std::move(v)), col(c)
    {
        if (!vec->type.is_vector() || col >= vec->type.dtypes.size()) throw std::runtime_error("length: bad column");
    }
};

// op_to_loop.h:106-119: probe of the vector's hash index on its iterator column; -1 on miss
struct Locate : ExprNode {
    Expr vec, iter;
    Locate(Expr v, Expr i) : ExprNode(types::IDX_T, NodeKind::LOCATE), vec(std::move(v)), iter(std::move(i))
    {
        if (!vec->type.is_vector() || vec->type.dim > 2) throw std::runtime_error("locate: bad vector");
        if (vec->type.iterty() != iter->type) throw std::runtime_error("locate: iterator type mismatch");
    }
};

struct ReadData : ExprNode {
    Expr vec, idx;
    size_t col;
    ReadData(Expr v, Expr i, size_t c)
        : ExprNode(v->type.dtypes.at(c), NodeKind::READDATA), vec(std::move(v)), idx(std::move(i)), col(c)
    {
    }
};

struct Func {
    string name;
    Expr output;
    vector<Sym> inputs;
    SymTable tbl;
    bool is_kernel;
    Func(string n, Expr o, vector<Sym> in, SymTable t = {}, bool k = false)
        : name(std::move(n)), output(std::move(o)), inputs(std::move(in)), tbl(std::move(t)), is_kernel(k)
    {
    }
};

// ------------------------------------------------------------------------------------------
// Builder DSL (reffiner.h:34-187)
// ------------------------------------------------------------------------------------------
namespace reffiner {

template <typename T>
struct _expr;

Expr _nary2(MathOp op, Expr a, Expr b);
Expr _elem_expr(Expr v, Expr i);

template <typename T>
struct _expr : public shared_ptr<T> {
    _expr(shared_ptr<T> p) : shared_ptr<T>(std::move(p)) {}
    template <typename U>
    _expr(const _expr<U>& o) : shared_ptr<T>(std::static_pointer_cast<T>(o))
    {
    }
    _expr<ExprNode> operator+(Expr o) const { return _nary2(MathOp::ADD, *this, o); }
    _expr<ExprNode> operator-(Expr o) const { return _nary2(MathOp::SUB, *this, o); }
    _expr<ExprNode> operator*(Expr o) const { return _nary2(MathOp::MUL, *this, o); }
    _expr<ExprNode> operator/(Expr o) const { return _nary2(MathOp::DIV, *this, o); }
    _expr<ExprNode> operator%(Expr o) const { return _nary2(MathOp::MOD, *this, o); }
    _expr<ExprNode> operator<(Expr o) const { return _nary2(MathOp::LT, *this, o); }
    _expr<ExprNode> operator<=(Expr o) const { return _nary2(MathOp::LTE, *this, o); }
    _expr<ExprNode> operator>(Expr o) const { return _nary2(MathOp::GT, *this, o); }
    _expr<ExprNode> operator>=(Expr o) const { return _nary2(MathOp::GTE, *this, o); }
    _expr<ExprNode> operator==(Expr o) const { return _nary2(MathOp::EQ, *this, o); }
    _expr<ExprNode> operator&(Expr o) const { return _nary2(MathOp::AND, *this, o); }
    _expr<ExprNode> operator|(Expr o) const { return _nary2(MathOp::OR, *this, o); }
    _expr<ExprNode> operator[](size_t n) const { return _expr<ExprNode>(make_shared<Get>(*this, n)); }
    _expr<ExprNode> operator[](Expr it) const { return _elem_expr(*this, it); }
    _expr<ExprNode> operator[](std::initializer_list<Expr> it) const { return _elem_expr(*this, *it.begin()); }
};

inline DataType nary_type(MathOp op, const Expr& a)
{
    switch (op) {
        case MathOp::LT: case MathOp::LTE: case MathOp::GT: case MathOp::GTE: case MathOp::EQ:
        case MathOp::NOT: case MathOp::AND: case MathOp::OR: case MathOp::IMPLIES: case MathOp::IFF:
            return types::BOOL_T;
        default: return a->type;
    }
}
inline Expr _nary2(MathOp op, Expr a, Expr b)
{
    if (a->type != b->type) throw std::runtime_error(string("binary operands differ in type: ") + mathop_name(op));
    if ((op == MathOp::AND || op == MathOp::OR) && a->type != types::BOOL_T)
        throw std::runtime_error("logical operator over non-bool");
    if (op == MathOp::MOD && a->type.is_float()) throw std::runtime_error("mod over float");
    if (op == MathOp::POW && !a->type.is_float()) throw std::runtime_error("pow over non-float");
    return make_shared<NaryExpr>(nary_type(op, a), op, vector<Expr>{a, b});
}
inline Expr _nary1(MathOp op, Expr a)
{
    if (op == MathOp::NOT && a->type != types::BOOL_T) throw std::runtime_error("not over non-bool");
    if ((op == MathOp::CEIL || op == MathOp::FLOOR) && !a->type.is_float()) throw std::runtime_error("ceil/floor of int");
    return make_shared<NaryExpr>(nary_type(op, a), op, vector<Expr>{a});
}
inline Expr _elem_expr(Expr v, Expr i) { return make_shared<Element>(v, i); }

using E = _expr<ExprNode>;
inline E _add(Expr a, Expr b) { return _nary2(MathOp::ADD, a, b); }
inline E _sub(Expr a, Expr b) { return _nary2(MathOp::SUB, a, b); }
inline E _mul(Expr a, Expr b) { return _nary2(MathOp::MUL, a, b); }
inline E _div(Expr a, Expr b) { return _nary2(MathOp::DIV, a, b); }
inline E _max(Expr a, Expr b) { return _nary2(MathOp::MAX, a, b); }
inline E _min(Expr a, Expr b) { return _nary2(MathOp::MIN, a, b); }
inline E _mod(Expr a, Expr b) { return _nary2(MathOp::MOD, a, b); }
inline E _pow(Expr a, Expr b) { return _nary2(MathOp::POW, a, b); }
inline E _lt(Expr a, Expr b) { return _nary2(MathOp::LT, a, b); }
inline E _lte(Expr a, Expr b) { return _nary2(MathOp::LTE, a, b); }
inline E _gt(Expr a, Expr b) { return _nary2(MathOp::GT, a, b); }
inline E _gte(Expr a, Expr b) { return _nary2(MathOp::GTE, a, b); }
inline E _eq(Expr a, Expr b) { return _nary2(MathOp::EQ, a, b); }
inline E _and(Expr a, Expr b) { return _nary2(MathOp::AND, a, b); }
inline E _or(Expr a, Expr b) { return _nary2(MathOp::OR, a, b); }
inline E _not(Expr a) { return _nary1(MathOp::NOT, a); }
inline E _neg(Expr a) { return _nary1(MathOp::NEG, a); }
inline E _abs(Expr a) { return _nary1(MathOp::ABS, a); }
inline E _sqrt(Expr a) { return _nary1(MathOp::SQRT, a); }
inline E _ceil(Expr a) { return _nary1(MathOp::CEIL, a); }
inline E _floor(Expr a) { return _nary1(MathOp::FLOOR, a); }
inline E _sel(Expr c, Expr t, Expr f) { return E(make_shared<Select>(c, t, f)); }
inline E _cast(DataType t, Expr a) { return E(make_shared<Cast>(t, a)); }
inline E _get(Expr v, size_t c) { return E(make_shared<Get>(v, c)); }
inline E _new(vector<Expr> v) { return E(make_shared<New>(std::move(v))); }
inline E _op(vector<Sym> it, Expr p, vector<Expr> out) { return E(make_shared<Op>(std::move(it), p, std::move(out))); }
inline E _red(Expr v, InitFnTy init, AccFnTy acc) { return E(Reduce::make(v, init, acc)); }
inline E _in(Expr i, Expr v) { return E(make_shared<In>(i, v)); }
inline E _elem(Expr v, Expr i) { return E(make_shared<Element>(v, i)); }
inline E _subvec(Expr v, Expr s, Expr e) { return E(make_shared<SubVector>(v, s, e)); }
inline E _len(Expr v, size_t c) { return E(make_shared<Length>(v, c)); }
inline E _locate(Expr v, Expr i) { return E(make_shared<Locate>(v, i)); }
inline E _readdata(Expr v, Expr i, size_t c) { return E(make_shared<ReadData>(v, i, c)); }
inline _expr<SymNode> _sym(string n, DataType t) { return _expr<SymNode>(make_shared<SymNode>(n, t)); }
inline _expr<SymNode> _sym(string n, Expr e) { return _expr<SymNode>(make_shared<SymNode>(n, e)); }
inline shared_ptr<Func> _func(string n, Expr o, vector<Sym> in, SymTable t = {}, bool k = false)
{
    return make_shared<Func>(n, o, std::move(in), std::move(t), k);
}
inline E _const(DataType t, double v) { return E(make_shared<Const>(t, v)); }
inline E _i8(int8_t v) { return _const(types::INT8_T, v); }
inline E _i16(int16_t v) { return _const(types::INT16_T, v); }
inline E _i32(int32_t v) { return _const(types::INT32_T, v); }
inline E _i64(int64_t v) { return _const(types::INT64_T, (double)v); }
inline E _u8(uint8_t v) { return _const(types::UINT8_T, v); }
inline E _u16(uint16_t v) { return _const(types::UINT16_T, v); }
inline E _u32(uint32_t v) { return _const(types::UINT32_T, v); }
inline E _u64(uint64_t v) { return _const(types::UINT64_T, (double)v); }
inline E _f32(float v) { return _const(types::FLOAT32_T, v); }
inline E _f64(double v) { return _const(types::FLOAT64_T, v); }
inline E _ch(char v) { return _const(types::INT8_T, v); }
inline E _idx(int64_t v) { return _const(types::IDX_T, (double)v); }
inline E _true() { return _const(types::BOOL_T, 1); }
inline E _false() { return _const(types::BOOL_T, 0); }

static const DataType _i8_t = types::INT8_T;
static const DataType _i16_t = types::INT16_T;
static const DataType _i32_t = types::INT32_T;
static const DataType _i64_t = types::INT64_T;
static const DataType _u8_t = types::UINT8_T;
static const DataType _u16_t = types::UINT16_T;
static const DataType _u32_t = types::UINT32_T;
static const DataType _u64_t = types::UINT64_T;
static const DataType _f32_t = types::FLOAT32_T;
static const DataType _f64_t = types::FLOAT64_T;
static const DataType _ch_t = types::INT8_T;
static const DataType _idx_t = types::IDX_T;
static const DataType _bool_t = types::BOOL_T;
template <size_t dim, typename... Ts>
DataType _vec_t()
{
    return types::VEC<dim, Ts...>();
}
template <typename... Ts>
DataType _struct_t()
{
    return types::STRUCT<Ts...>();
}

}  // namespace reffiner

// ------------------------------------------------------------------------------------------
// Text form
// ------------------------------------------------------------------------------------------
inline string fmt_double(double v)
{
    if (std::isnan(v)) return "nan";
    if (std::isinf(v)) return v > 0 ? "inf" : "-inf";
    char buf[64];
    snprintf(buf, sizeof buf, "%.17g", v);
    return buf;
}

class Printer {
public:
    explicit Printer(const Func& fn) : fn_(fn) {}
    string run()
    {
        for (auto& s : fn_.inputs) name(s);
        for (auto& kv : fn_.tbl) name(kv.first);
        std::ostringstream o;
        o << "(func " << fn_.name << " " << e(fn_.output) << " (inputs";
        for (auto& s : fn_.inputs) o << " (" << name(s) << " " << s->type.str() << ")";
        o << ") (tbl";
        for (auto& kv : fn_.tbl) o << " (" << name(kv.first) << " " << e(kv.second) << ")";
        o << "))";
        return o.str();
    }

private:
    string name(const Sym& s)
    {
        auto it = names_.find(s.get());
        if (it != names_.end()) return it->second;
        string base;
        for (char c : s->name) base += (isalnum((unsigned char)c) || c == '_' || c == '.' || c == '$') ? c : '_';
        if (base.empty()) base = "sym";
        string nm = base;
        for (int i = 1; used_.count(nm); i++) nm = base + "#" + std::to_string(i);
        used_[nm] = 1;
        names_[s.get()] = nm;
        return nm;
    }
    string e(const Expr& x)
    {
        switch (x->kind) {
            case NodeKind::SYM: return name(std::static_pointer_cast<SymNode>(x));
            case NodeKind::CONST: {
                auto c = (const Const*)x.get();
                return "(const " + c->type.str() + " " + fmt_double(c->val) + ")";
            }
            case NodeKind::NARY: {
                auto n = (const NaryExpr*)x.get();
                string s = string("(") + mathop_name(n->op);
                for (auto& a : n->args) s += " " + e(a);
                return s + ")";
            }
            case NodeKind::SELECT: {
                auto n = (const Select*)x.get();
                return "(sel " + e(n->cond) + " " + e(n->true_body) + " " + e(n->false_body) + ")";
            }
            case NodeKind::CAST: {
                auto n = (const Cast*)x.get();
                return "(cast " + n->type.str() + " " + e(n->arg) + ")";
            }
            case NodeKind::GET: {
                auto n = (const Get*)x.get();
                return "(get " + e(n->val) + " " + std::to_string(n->col) + ")";
            }
            case NodeKind::NEW: {
                auto n = (const New*)x.get();
                string s = "(new";
                for (auto& v : n->vals) s += " " + e(v);
                return s + ")";
            }
            case NodeKind::OP: {
                auto n = (const Op*)x.get();
                string s = "(op (";
                for (size_t i = 0; i < n->iters.size(); i++)
                    s += (i ? " (" : "(") + name(n->iters[i]) + " " + n->iters[i]->type.str() + ")";
                s += ") " + e(n->pred) + " (";
                for (size_t i = 0; i < n->outputs.size(); i++) s += (i ? " " : "") + e(n->outputs[i]);
                return s + "))";
            }
            case NodeKind::ELEMENT: {
                auto n = (const Element*)x.get();
                return "(elem " + e(n->vec) + " " + e(n->iter) + ")";
            }
            case NodeKind::IN: {
                auto n = (const In*)x.get();
                return "(in " + e(n->iter) + " " + e(n->vec) + ")";
            }
            case NodeKind::REDUCE: {
                auto n = (const Reduce*)x.get();
                return "(reduce " + e(n->vec) + " " + e(n->init_expr) + " (" + name(n->state) + " " +
                       n->state->type.str() + ") (" + name(n->val) + " " + n->val->type.str() + ") " + e(n->acc_expr) +
                       ")";
            }
            case NodeKind::SUBVECTOR: {
                auto n = (const SubVector*)x.get();
                return "(subvec " + e(n->vec) + " " + e(n->start) + " " + e(n->end) + ")";
            }
            case NodeKind::LENGTH: {
                auto n = (const Length*)x.get();
                return "(len " + e(n->vec) + " " + std::to_string(n->col) + ")";
            }
            case NodeKind::LOCATE: {
                auto n = (const Locate*)x.get();
                return "(locate " + e(n->vec) + " " + e(n->iter) + ")";
            }
            case NodeKind::READDATA: {
                auto n = (const ReadData*)x.get();
                return "(readdata " + e(n->vec) + " " + e(n->idx) + " " + std::to_string(n->col) + ")";
            }
        }
        throw std::runtime_error("unprintable node");
    }
    const Func& fn_;
    std::unordered_map<const void*, string> names_;
    std::map<string, int> used_;
};

inline string to_text(const Func& fn) { return Printer(fn).run(); }

// S-expression reader producing the same nodes.  Symbols are resolved by name: function inputs,
// table entries, op iterators and reduce state/value symbols (the latter two are scoped).
class Parser {
public:
    explicit Parser(const string& text) : s_(text) {}

    shared_ptr<Func> parse()
    {
        auto root = read();
        if (!root.list || root.items.size() != 5 || root.items[0].atom != "func")
            throw std::runtime_error("expected (func NAME OUTPUT (inputs ...) (tbl ...))");
        auto& inputs = root.items[3];
        auto& tbl = root.items[4];
        if (!inputs.list || inputs.items.empty() || inputs.items[0].atom != "inputs") throw std::runtime_error("bad inputs");
        if (!tbl.list || tbl.items.empty() || tbl.items[0].atom != "tbl") throw std::runtime_error("bad tbl");
        declare(root.items[2]);
        for (size_t i = 1; i < tbl.items.size(); i++) declare(tbl.items[i].at(1));
        vector<Sym> ins;
        for (size_t i = 1; i < inputs.items.size(); i++) {
            auto& d = inputs.items[i];
            auto sym = make_shared<SymNode>(d.at(0).atom, type(d.at(1)));
            syms_[sym->name] = sym;
            ins.push_back(sym);
        }
        // table symbols: types come from their expressions, which may reference other table
        // symbols; resolve lazily
        for (size_t i = 1; i < tbl.items.size(); i++) pending_[tbl.items[i].at(0).atom] = &tbl.items[i].at(1);
        SymTable t;
        for (size_t i = 1; i < tbl.items.size(); i++) {
            auto nm = tbl.items[i].at(0).atom;
            auto sym = table_sym(nm);
            t[sym] = defs_.at(nm);
        }
        auto out = expr(root.items[2]);
        return make_shared<Func>(root.items[1].atom, out, ins, t);
    }

private:
    struct Node {
        bool list = false;
        string atom;
        vector<Node> items;
        const Node& at(size_t i) const
        {
            if (!list || i >= items.size()) throw std::runtime_error("malformed expression near '" + atom + "'");
            return items[i];
        }
    };
    Node read()
    {
        skip();
        if (p_ >= s_.size()) throw std::runtime_error("unexpected end of text");
        Node n;
        if (s_[p_] == '(') {
            n.list = true;
            p_++;
            for (;;) {
                skip();
                if (p_ >= s_.size()) throw std::runtime_error("unbalanced parentheses");
                if (s_[p_] == ')') {
                    p_++;
                    break;
                }
                n.items.push_back(read());
            }
            return n;
        }
        size_t b = p_;
        while (p_ < s_.size() && !isspace((unsigned char)s_[p_]) && s_[p_] != '(' && s_[p_] != ')') p_++;
        n.atom = s_.substr(b, p_ - b);
        return n;
    }
    void skip()
    {
        while (p_ < s_.size() && isspace((unsigned char)s_[p_])) p_++;
    }
    DataType type(const Node& n)
    {
        if (!n.list) {
            static const std::map<string, BaseType> m = {
                {"bool", BOOL}, {"i8", INT8}, {"i16", INT16}, {"i32", INT32}, {"i64", INT64}, {"u8", UINT8},
                {"u16", UINT16}, {"u32", UINT32}, {"u64", UINT64}, {"f32", FLOAT32}, {"f64", FLOAT64},
                {"idx", IDX}, {"void", VOID}};
            auto it = m.find(n.atom);
            if (it == m.end()) throw std::runtime_error("unknown type " + n.atom);
            return DataType(it->second);
        }
        auto& h = n.at(0).atom;
        if (h == "struct") {
            vector<DataType> d;
            for (size_t i = 1; i < n.items.size(); i++) d.push_back(type(n.items[i]));
            return DataType(STRUCT, d);
        }
        if (h == "vector") {
            size_t dim = std::stoul(n.at(1).atom);
            vector<DataType> d;
            for (auto& c : n.at(2).items) d.push_back(type(c));
            vector<EncodeType> e;
            for (auto& c : n.at(3).items) e.push_back(c.atom == "runend" ? RUNEND : FLAT);
            return DataType(VECTOR, d, dim, e);
        }
        throw std::runtime_error("unknown type form " + h);
    }
    // op iterators and reduce state/value symbols carry unique names in the text; declare them
    // up front because table entries evaluated inside an op refer to its iterators
    void declare(const Node& n)
    {
        if (!n.list || n.items.empty()) return;
        const string& h = n.items[0].atom;
        if (h == "op" && n.items.size() > 1) {
            for (auto& d : n.at(1).items) bound_[d.at(0).atom] = make_shared<SymNode>(d.at(0).atom, type(d.at(1)));
        } else if (h == "reduce" && n.items.size() > 4) {
            for (int k = 3; k <= 4; k++)
                bound_[n.at(k).at(0).atom] = make_shared<SymNode>(n.at(k).at(0).atom, type(n.at(k).at(1)));
        }
        for (auto& c : n.items) declare(c);
    }
    Sym table_sym(const string& nm)
    {
        auto it = syms_.find(nm);
        if (it != syms_.end()) return it->second;
        if (in_progress_.count(nm)) throw std::runtime_error("cyclic symbol definition " + nm);
        in_progress_[nm] = 1;
        auto def = expr(*pending_.at(nm));
        in_progress_.erase(nm);
        auto sym = make_shared<SymNode>(nm, def->type);
        syms_[nm] = sym;
        defs_[nm] = def;
        return sym;
    }
    Sym lookup(const string& nm)
    {
        auto b = bound_.find(nm);
        if (b != bound_.end()) return b->second;
        auto f = syms_.find(nm);
        if (f != syms_.end()) return f->second;
        if (pending_.count(nm)) return table_sym(nm);
        throw std::runtime_error("unknown symbol " + nm);
    }
    static MathOp opcode(const string& h, bool& ok)
    {
        static const std::map<string, MathOp> m = {
            {"add", MathOp::ADD}, {"sub", MathOp::SUB}, {"mul", MathOp::MUL}, {"div", MathOp::DIV},
            {"max", MathOp::MAX}, {"min", MathOp::MIN}, {"mod", MathOp::MOD}, {"sqrt", MathOp::SQRT},
            {"pow", MathOp::POW}, {"abs", MathOp::ABS}, {"neg", MathOp::NEG}, {"ceil", MathOp::CEIL},
            {"floor", MathOp::FLOOR}, {"lt", MathOp::LT}, {"lte", MathOp::LTE}, {"gt", MathOp::GT},
            {"gte", MathOp::GTE}, {"eq", MathOp::EQ}, {"not", MathOp::NOT}, {"and", MathOp::AND},
            {"or", MathOp::OR}};
        auto it = m.find(h);
        ok = it != m.end();
        return ok ? it->second : MathOp::ADD;
    }
    Expr expr(const Node& n)
    {
        if (!n.list) return lookup(n.atom);
        const string& h = n.at(0).atom;
        bool isop = false;
        MathOp op = opcode(h, isop);
        if (isop) {
            if (n.items.size() == 2) return reffiner::_nary1(op, expr(n.items[1]));
            if (n.items.size() == 3) return reffiner::_nary2(op, expr(n.items[1]), expr(n.items[2]));
            throw std::runtime_error("bad arity for " + h);
        }
        if (h == "const") {
            string v = n.at(2).atom;
            double d = v == "nan" ? NAN : v == "inf" ? INFINITY : v == "-inf" ? -INFINITY : std::strtod(v.c_str(), nullptr);
            return make_shared<Const>(type(n.at(1)), d);
        }
        if (h == "sel") return make_shared<Select>(expr(n.at(1)), expr(n.at(2)), expr(n.at(3)));
        if (h == "cast") return make_shared<Cast>(type(n.at(1)), expr(n.at(2)));
        if (h == "get") return make_shared<Get>(expr(n.at(1)), std::stoul(n.at(2).atom));
        if (h == "new") {
            vector<Expr> v;
            for (size_t i = 1; i < n.items.size(); i++) v.push_back(expr(n.items[i]));
            return make_shared<New>(v);
        }
        if (h == "op") {
            vector<Sym> iters;
            for (auto& d : n.at(1).items) iters.push_back(bound_.at(d.at(0).atom));
            auto pred = expr(n.at(2));
            vector<Expr> outs;
            for (auto& o : n.at(3).items) outs.push_back(expr(o));
            return make_shared<Op>(iters, pred, outs);
        }
        if (h == "reduce") {
            auto vec = expr(n.at(1));
            auto init = expr(n.at(2));
            auto st = bound_.at(n.at(3).at(0).atom);
            auto vl = bound_.at(n.at(4).at(0).atom);
            auto acc = expr(n.at(5));
            return make_shared<Reduce>(vec, init, st, vl, acc);
        }
        if (h == "elem") return make_shared<Element>(expr(n.at(1)), expr(n.at(2)));
        if (h == "in") return make_shared<In>(expr(n.at(1)), expr(n.at(2)));
        if (h == "subvec") return make_shared<SubVector>(expr(n.at(1)), expr(n.at(2)), expr(n.at(3)));
        if (h == "len") return make_shared<Length>(expr(n.at(1)), std::stoul(n.at(2).atom));
        if (h == "locate") return make_shared<Locate>(expr(n.at(1)), expr(n.at(2)));
        if (h == "readdata") return make_shared<ReadData>(expr(n.at(1)), expr(n.at(2)), std::stoul(n.at(3).atom));
        throw std::runtime_error("unknown node " + h);
    }

    string s_;
    size_t p_ = 0;
    std::map<string, Sym> syms_;
    std::map<string, Expr> defs_;
    std::map<string, const Node*> pending_;
    std::map<string, int> in_progress_;
    std::map<string, Sym> bound_;
};

inline shared_ptr<Func> parse_text(const string& text) { return Parser(text).parse(); }

}  // namespace reffine
