"""Arrow IPC ingest without a GPU: the library's own parser (rf_ipc_read) against fixtures
written by pyarrow (tests/golden/make_ipc.py), and its refusals of damaged or unsupported files."""
import os
import shutil

import numpy as np
import pytest

from reffine_gb300 import _capi, ir, workloads as W
from reffine_gb300.ipc_write import write_ipc
from reffine_gb300.table import Table, read_ipc_c, release_c, table_from_ipc, unpack_validity

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_filter_sum_columns_and_type():
    t = table_from_ipc(os.path.join(GOLDEN, "ipc_filter_sum.arrow"), 2)
    ref = np.load(os.path.join(GOLDEN, "ipc_filter_sum.npz"))
    assert [c.name for c in t.columns] == list(ref.files)
    for c in t.columns:
        assert np.array_equal(c.data, ref[c.name]) and c.data.dtype == ref[c.name].dtype
    ty = t.get_data_type()
    assert ty.dim == 2 and [str(d) for d in ty.dtypes] == ["i64", "i32", "f64", "f64", "f64"]


def test_every_width_with_nulls():
    t = table_from_ipc(os.path.join(GOLDEN, "ipc_types.arrow"), 1)
    ref = np.load(os.path.join(GOLDEN, "ipc_types.npz"))
    for c in t.columns:
        valid = unpack_validity(c.valid, len(c.data))
        assert np.array_equal(valid, ref["valid_" + c.name]), c.name
        # values under a null are unspecified; compare the valid ones
        assert np.array_equal(c.data[valid], ref[c.name][valid]), c.name
        assert c.data.dtype == ref[c.name].dtype


def test_run_end_encoded_column():
    t = table_from_ipc(os.path.join(GOLDEN, "ipc_runend.arrow"), 2)
    ref = np.load(os.path.join(GOLDEN, "ipc_runend.npz"))
    key, val = t.columns
    assert key.encoding == ir.RUNEND
    assert np.array_equal(key.run_ends, ref["run_ends"]) and np.array_equal(key.data, ref["run_values"])
    assert np.array_equal(val.data, ref["value"]) and len(t) == len(ref["keys"])


def test_c_data_release_frees_once():
    s, a = read_ipc_c(os.path.join(GOLDEN, "ipc_runend.arrow"))
    assert s.format == b"+s" and s.n_children == 2 and a.n_children == 2
    assert s.children[0].contents.format == b"+r"
    release_c(s, a)
    assert not s.release and not a.release


@pytest.mark.parametrize("name,status,msg", [("ipc_lz4", _capi.RF_ERR_UNSUPPORTED, "compressed"),
                                             ("ipc_dict", _capi.RF_ERR_UNSUPPORTED, "dictionary")])
def test_unsupported_files_are_refused(name, status, msg):
    with pytest.raises(_capi.RfError) as e:
        read_ipc_c(os.path.join(GOLDEN, name + ".arrow"))
    assert e.value.status == status and msg in str(e.value)


def test_damaged_files_fail_cleanly(tmp_path):
    src = open(os.path.join(GOLDEN, "ipc_types.arrow"), "rb").read()
    cases = {"empty": b"", "magic": b"XXXXXX" + src[6:], "truncated": src[: len(src) // 2],
             "tail": src[:-3]}
    # flipped bytes across the footer and the message metadata: every one is an error or a valid
    # read, never a crash
    rng = np.random.default_rng(1)
    for i, pos in enumerate(rng.integers(len(src) - 600, len(src) - 6, 60)):
        b = bytearray(src)
        b[pos] ^= 0xFF
        cases["flip%d" % i] = bytes(b)
    for name, data in cases.items():
        p = tmp_path / (name + ".arrow")
        p.write_bytes(data)
        try:
            s, a = read_ipc_c(str(p))
            release_c(s, a)
        except _capi.RfError as e:
            assert e.status in (_capi.RF_ERR_INVALID, _capi.RF_ERR_UNSUPPORTED)
    with pytest.raises(_capi.RfError, match="cannot open"):
        read_ipc_c(str(tmp_path / "missing.arrow"))


def _types_table():
    ref = np.load(os.path.join(GOLDEN, "ipc_types.npz"))
    names = [n for n in ref.files if not n.startswith("valid_")]
    return Table.from_arrays(1, {n: ref[n] for n in names}, valid={n: ref["valid_" + n] for n in names}), ref, names


def test_writer_round_trips_through_own_reader(tmp_path):
    # every width with nulls, and a run-end column: written by ipc_write, read by rf_ipc_read
    t, ref, names = _types_table()
    p = str(tmp_path / "types.arrow")
    write_ipc(p, t)
    back = table_from_ipc(p, 1)
    for c, n in zip(back.columns, names):
        m = unpack_validity(c.valid, len(c.data))
        assert np.array_equal(m, ref["valid_" + n]) and np.array_equal(c.data[m], ref[n][m]), n
        assert c.dtype == t.columns[names.index(n)].dtype
    ree = W.ree_sorted(W.hashgroup_table(20_000, 700, 1.1, seed=8))
    p = str(tmp_path / "ree.arrow")
    write_ipc(p, ree)
    back = table_from_ipc(p, 2)
    assert back.columns[0].encoding == ir.RUNEND
    assert np.array_equal(back.columns[0].run_ends, ree.columns[0].run_ends)
    assert np.array_equal(back.columns[0].data, ree.columns[0].data)
    assert np.array_equal(back.columns[1].data, ree.columns[1].data)


def test_writer_output_is_valid_arrow(tmp_path):
    pa = pytest.importorskip("pyarrow")
    ipc = pytest.importorskip("pyarrow.ipc")
    t, ref, names = _types_table()
    p = str(tmp_path / "types.arrow")
    write_ipc(p, t)
    b = ipc.open_file(p).get_batch(0)
    b.validate(full=True)
    for n in names:
        col = b.column(n)
        m = ~col.is_null().to_numpy(zero_copy_only=False)
        assert np.array_equal(m, ref["valid_" + n])
        assert np.array_equal(col.to_numpy(zero_copy_only=False)[m], ref[n][m]), n
    ree = W.ree_sorted(W.hashgroup_table(3_000, 100, 1.1, seed=9))
    write_ipc(p, ree)
    b = ipc.open_file(p).get_batch(0)
    b.validate(full=True)
    assert isinstance(b.column(0), pa.RunEndEncodedArray) and b.num_rows == 3_000
