"""Arrow IPC fixtures for the ingest tests (rf_ipc_read / rf_table_load_ipc), written with
pyarrow in the build container (the GPU machine has no pyarrow).  Each file has an .npz beside it
holding the same columns as numpy arrays (and validity masks / run ends) for the comparison.

    python tests/golden/make_ipc.py
"""
import os

import numpy as np
import pyarrow as pa
import pyarrow.ipc as ipc

HERE = os.path.dirname(os.path.abspath(__file__))


def write(name, batch, arrays, options=None):
    with pa.OSFile(os.path.join(HERE, name + ".arrow"), "wb") as f:
        with ipc.new_file(f, batch.schema, options=options) as w:
            w.write_batch(batch)
    if arrays is not None:
        np.savez(os.path.join(HERE, name + ".npz"), **arrays)


def main():
    rng = np.random.default_rng(7)
    # the filter+sum shape (dim 2: key, day, price, discount, quantity)
    n = 5_003
    fs = {"key": np.arange(n, dtype=np.int64), "day": rng.integers(0, 2557, n, dtype=np.int32),
          "price": rng.uniform(900.0, 105000.0, n), "discount": rng.integers(0, 11, n) / 100.0,
          "quantity": rng.integers(1, 51, n).astype(np.float64)}
    write("ipc_filter_sum", pa.record_batch([pa.array(v) for v in fs.values()], names=list(fs)), fs)
    # every supported width, with nulls
    m = 1_001
    cols = {"i8": rng.integers(-100, 100, m, dtype=np.int8), "u8": rng.integers(0, 250, m, dtype=np.uint8),
            "i16": rng.integers(-30000, 30000, m, dtype=np.int16), "i32": rng.integers(-2**31, 2**31 - 1, m, dtype=np.int32),
            "u32": rng.integers(0, 2**32 - 1, m, dtype=np.uint32), "i64": rng.integers(-2**62, 2**62, m, dtype=np.int64),
            "f32": rng.standard_normal(m).astype(np.float32), "f64": rng.standard_normal(m)}
    masks = {k: rng.random(m) < 0.9 for k in cols}
    arrs = [pa.array(v, mask=~masks[k]) for k, v in cols.items()]
    out = dict(cols)
    out.update({"valid_" + k: v for k, v in masks.items()})
    write("ipc_types", pa.record_batch(arrs, names=list(cols)), out)
    # a run-end encoded key column (the multidim shape: sorted keys, runs, one value per row)
    keys = np.sort(rng.integers(0, 300, 4_000)).astype(np.int64)
    vals = rng.uniform(0.0, 100.0, len(keys))
    run_vals, starts = np.unique(keys, return_index=True)
    run_ends = np.append(starts[1:], len(keys)).astype(np.int32)
    ree = pa.RunEndEncodedArray.from_arrays(pa.array(run_ends, pa.int32()), pa.array(run_vals, pa.int64()))
    write("ipc_runend", pa.record_batch([ree, pa.array(vals)], names=["key", "value"]),
          {"run_ends": run_ends, "run_values": run_vals, "keys": keys, "value": vals})
    # refused: a compressed body, a dictionary column
    small = pa.record_batch([pa.array(np.arange(100, dtype=np.int64))], names=["a"])
    write("ipc_lz4", small, None, ipc.IpcWriteOptions(compression="lz4"))
    dict_col = pa.array(["x", "y", "x"]).dictionary_encode()
    write("ipc_dict", pa.record_batch([dict_col], names=["d"]), None)


if __name__ == "__main__":
    main()
