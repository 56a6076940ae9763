// Stand-in for Reffine's printer2.h (which needs LLVM): only what src/ir/ir.cpp uses, so that
// Reffine's IR, builder and pass sources compile with g++ alone.  ExprNode::str() prints through
// it (src/ir/ir.cpp:54-58), and Reffine's passes name a few symbols from it (a vector's length
// symbol is `<vector name>_len`, include/reffine/iter/iter_space.h:112), so a symbol prints as
// its name, as IRPrinter2::visit(Sym) does for a symbol with no definition
// (src/pass/printer2.cpp:13-15).  Any other expression prints as a placeholder; Reffine uses those
// strings only as the names of output columns.
#pragma once
#include <memory>
#include <string>

#include "reffine/ir/node.h"

namespace reffine {
struct IRPrinter2 {
    static std::string Build(Expr e)
    {
        if (auto s = std::dynamic_pointer_cast<SymNode>(e)) return s->name;
        return "<expr>";
    }
};
}  // namespace reffine
