// The table handle Reffine's generated query functions take: `ArrowTable*`.
//
// Same declaration as Reffine's (include/reffine/arrow/abi.h:56-69): a polymorphic struct
// {dim, schema, array, index}.  Keeping the declaration identical keeps the object layout
// identical, so tables built by code written against Reffine (ArrowTable2 and friends) can be
// passed to this backend's query functions unchanged.
#pragma once

#include <cstdint>
#include <unordered_map>

#include "reffine_gb300/arrow_c.h"

using IndexTy = std::unordered_map<int64_t, int64_t>;

extern "C" {
struct ArrowTable {
    int64_t dim;
    ArrowSchema* schema;
    ArrowArray* array;
    IndexTy* index;

    ArrowTable(int64_t dim, ArrowSchema* schema = nullptr, ArrowArray* array = nullptr)
        : dim(dim), schema(schema), array(array), index(nullptr)
    {
    }

    virtual ~ArrowTable() {}
};
}
