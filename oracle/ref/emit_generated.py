#!/usr/bin/env python3
"""Writes oracle/ref/generated/<query>.cpp: the C++ that Reffine's own compile path emits for the
four benchmark query shapes, so that the CPU reference arm can run Reffine's generated code where
no Reffine checkout is at hand (the GPU machine).  Test and benchmark infrastructure only.

    python oracle/ref/emit_generated.py [REFFINE_SRC]      (default: /root/reference)

The text is what oracle/ref_pipeline.py's emit() returns for compile_op's default mode
(vectorize off, include/reffine/utils/utils.h:47-54, as Reffine's benchmarks call it), with one
change: CEmitter names temporaries after heap addresses (`lb_0x27f9dc10`), which differ from run
to run, so each address is renumbered in order of first appearance, and an output's builder
number (which counts the queries emitted before it in the process) is written as 0.  The code includes
"reffine/vinstr/vinstr.h"; oracle/ref/runtime provides that interface for it.
"""
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
GEN_DIR = os.path.join(HERE, "generated")
QUERIES = ["filter_sum", "groupby", "join_agg", "hashgroup_ree"]


def normalise(code: str) -> str:
    ids = {}

    def sub(m):
        a = m.group(0)
        if a not in ids:
            ids[a] = "n%d" % len(ids)
        return ids[a]

    code = re.sub(r"0x[0-9a-f]{4,}", sub, code)
    # make_vector's second argument numbers the output builders Reffine registered in this
    # process so far (src/engine/memory.cpp:5-9); the emitted query makes one output, so it is 0
    return re.sub(r"make_vector\((int64_t\(\d+\)), uint32_t\(\d+\)\)", r"make_vector(\1, uint32_t(0))", code)


def generate(name: str) -> str:
    from oracle import ref_pipeline as RP
    code, sym = RP.emit(name, False)
    head = ("// Emitted by Reffine's compile path (LoopGen, CanonPass, ReadWritePass, ScalarPass,\n"
            "// CEmitter) for query `%s` of oracle/ref/ref_queries.h, vectorize off; temporaries\n"
            "// named after heap addresses renumbered.  Regenerate with oracle/ref/emit_generated.py.\n"
            "// entry: %s\n" % (name, sym))
    return head + normalise(code)


def main():
    sys.path.insert(0, ROOT)
    sys.path.insert(0, HERE)
    from build_ref import build
    build(sys.argv[1] if len(sys.argv) > 1 else "/root/reference", quiet=True)
    os.makedirs(GEN_DIR, exist_ok=True)
    for q in QUERIES:
        with open(os.path.join(GEN_DIR, q + ".cpp"), "w") as f:
            f.write(generate(q))
        print("wrote", os.path.join(GEN_DIR, q + ".cpp"))


if __name__ == "__main__":
    main()
