"""Arrow IPC ingest without a GPU: the library's own parser (rf_ipc_read) against fixtures
written by pyarrow (tests/golden/make_ipc.py), and its refusals of damaged or unsupported files."""
import os
import shutil

import numpy as np
import pytest

from reffine_gb300 import _capi, ir
from reffine_gb300.table import read_ipc_c, release_c, table_from_ipc, unpack_validity

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
