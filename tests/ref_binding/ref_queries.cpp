// Test program: the queries of oracle/ref/ref_queries.h (built with Reffine's own IR builder),
// printed by the GPU backend's binding (reffine_gb300::func_text) one per line as NAME<TAB>TEXT.
// tests/test_ref_binding.py checks that each text is the expression graph the Python builder
// makes for the same query.  Built only where Reffine's headers and builder sources are available.
#include <cstdio>

#include "ref_queries.h"
#include "reffine_gb300/ref_binding.h"

int main()
{
    for (auto& [name, make] : refq::queries()) {
        auto fn = make();
        printf("%s\t%s\n", name, reffine_gb300::func_text(*fn).c_str());
    }
    return 0;
}
