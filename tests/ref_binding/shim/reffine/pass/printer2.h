// Stand-in for Reffine's printer2.h (which needs LLVM): only what src/ir/ir.cpp uses, so the
// reference's IR and builder sources compile with g++ alone for the binding's test program.
#pragma once
#include <string>

#include "reffine/ir/node.h"

namespace reffine {
struct IRPrinter2 {
    static std::string Build(Expr) { return "<expr>"; }
};
}  // namespace reffine
