#!/usr/bin/env python3
"""Writes tests/golden/ref_pipeline.json and ref_pipeline_hashgroup.npz: the answers of Reffine's
own compile path (oracle/ref_pipeline.py: Reffine's LoopGen, CanonPass, ReadWritePass, ScalarPass
and CEmitter, the emitted C++ compiled with g++) for the four benchmark query shapes on seeded
tables.  The tests compare the oracle and the GPU with these answers where no Reffine checkout is
at hand.

    python tests/golden/make_ref_pipeline_golden.py REFFINE_SRC

REFFINE_SRC is a Reffine checkout; oracle/ref/build_ref.py builds the pipeline from it.  Each
query runs in both vectorize modes and in two floating-point builds of the emitted code:
``exact`` (-ffp-contract=off: every product rounded before it is added) and ``fma`` (a*b + c
fused, as clang's default contraction with Reffine's host-targeted JIT gives on a CPU with FMA).
The tables are regenerated from their seeds by reffine_gb300.workloads; a SHA-256 of each
table's columns is stored beside the answers so that a change of generator shows.
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from reffine_gb300 import workloads as W  # noqa: E402

OUT_JSON = os.path.join(HERE, "ref_pipeline.json")
OUT_NPZ = os.path.join(HERE, "ref_pipeline_hashgroup.npz")


def cases():
    """name -> (ref query name, Python-built Func, tables, table recipe)."""
    fs = W.filter_sum_table(200_003, seed=11)
    gb = W.groupby_table(300_007, seed=12)
    b, p = W.join_tables(20_000, 300_007, seed=13)
    hg = W.ree_sorted(W.hashgroup_table(100_003, 10_000, 1.1, seed=14))
    return {
        "filter_sum": ("filter_sum", W.filter_sum_query(fs.get_data_type()), [fs],
                       "filter_sum_table(200003, seed=11)"),
        "groupby": ("groupby", W.groupby_query(gb.get_data_type()), [gb], "groupby_table(300007, seed=12)"),
        "join_agg": ("join_agg", W.join_query(b.get_data_type(), p.get_data_type()), [b, p],
                     "join_tables(20000, 300007, seed=13)"),
        "hashgroup_ree": ("hashgroup_ree", W.hashgroup_query(hg.get_data_type()), [hg],
                          "ree_sorted(hashgroup_table(100003, 10000, 1.1, seed=14))"),
    }


def table_digest(tables) -> str:
    h = hashlib.sha256()
    for t in tables:
        for c in t.columns:
            h.update(c.data.tobytes())
            if c.valid is not None:
                h.update(c.valid.tobytes())
            if c.run_ends is not None:
                h.update(c.run_ends.tobytes())
    return h.hexdigest()


def encode(v):
    """A value result as JSON: floats as exact hex strings."""
    if isinstance(v, (tuple, list)):
        return [encode(x) for x in v]
    if isinstance(v, float):
        return {"f": float.hex(v)}
    return int(v)


def decode(v):
    if isinstance(v, list):
        return tuple(decode(x) for x in v)
    if isinstance(v, dict):
        return float.fromhex(v["f"])
    return v


def main():
    if len(sys.argv) < 2:
        raise SystemExit(__doc__)
    sys.path.insert(0, os.path.join(ROOT, "oracle", "ref"))
    from build_ref import build
    build(sys.argv[1])
    from oracle import ref_pipeline as RP
    out = {"cases": {}}
    arrays = {}
    for name, (qname, fn, tables, recipe) in cases().items():
        entry = {"tables": recipe, "sha256": table_digest(tables), "results": {}}
        for vec in (False, True):
            for mode, contract in (("exact", False), ("fma", True)):
                r = RP.RefQuery(qname, fn, vec, contract)(*tables)
                key = "%s_%s" % ("vectorize" if vec else "scalar", mode)
                if isinstance(r, dict):
                    # columns stored once per distinct content (keys and counts agree across builds)
                    names = []
                    for col in r["cols"]:
                        nm = "a_" + hashlib.sha256(col.tobytes() + str(col.dtype).encode()).hexdigest()[:16]
                        arrays[nm] = col
                        names.append(nm)
                    entry["results"][key] = {"len": r["len"], "cols": names}
                else:
                    entry["results"][key] = encode(r)
        out["cases"][name] = entry
        print(name, "done")
    with open(OUT_JSON, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    np.savez_compressed(OUT_NPZ, **arrays)
    print("wrote %s and %s" % (OUT_JSON, OUT_NPZ))


if __name__ == "__main__":
    main()
