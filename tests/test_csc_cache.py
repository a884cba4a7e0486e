"""The reference's binary CSC matrix cache (ipt_block_csc_cache_*): files in
the layout its benchmarks write are read back exactly, files written here
parse with the reference's own inspection layout, and foreign or broken
files are rejected as the reference's reader rejects them."""
import numpy as np
import pytest

from block_ipt_gb300 import api
from oracle import oracle


def h2o(golden):
    arrays, _ = golden
    name = "h20_fci_w_k1"
    return (arrays["sparse_%s_col_ptr" % name], arrays["sparse_%s_row_ind" % name],
            arrays["sparse_%s_values_csc" % name])


def diag_of(cp, ri, va):
    n = len(cp) - 1
    d = np.zeros(n)
    for c in range(n):
        for p in range(cp[c], cp[c + 1]):
            if ri[p] == c:
                d[c] = va[p]
                break
    return d


def test_reads_reference_layout(lib, golden, tmp_path):
    cp, ri, va = h2o(golden)
    dg = diag_of(cp, ri, va)
    path = tmp_path / "h2o.bin"
    path.write_bytes(oracle.reference_csc_cache_bytes(b"IPTH2OC1", cp, ri, va, dg, 12.5,
                                                      (7, 10, 5, 5, 21, 21)))
    rcp, rri, rva, rdg, meta = api.read_csc_cache(str(path))
    np.testing.assert_array_equal(rcp, cp)
    np.testing.assert_array_equal(rri, ri)
    assert np.array_equal(rva.view(np.uint64), np.asarray(va, np.float64).view(np.uint64))
    np.testing.assert_array_equal(rdg, dg)
    assert meta["magic"] == "IPTH2OC1" and meta["version"] == 1 and meta["n"] == len(cp) - 1
    assert meta["matrix_inf_norm"] == 12.5
    assert [meta[f] for f in ("norb", "nelec", "neleca", "nelecb", "na", "nb")] == \
        [7, 10, 5, 5, 21, 21]


def test_written_files_parse_with_reference_layout(lib, tmp_path):
    cp, ri, va, H = oracle.cluster_test_matrix(70, 4, 0.2)
    dg = np.diag(H).copy()
    path = tmp_path / "gen.bin"
    api.write_csc_cache(str(path), cp, ri, va, dg, magic="IPTCH4C1", norb=8, nelec=8,
                        neleca=4, nelecb=4, na=70, nb=1)
    data = path.read_bytes()
    ref = oracle.parse_reference_csc_cache(data)
    assert len(data) == 56 + 4 * (70 + 1) + 12 * len(ri) + 8 * 70
    assert ref["magic"] == "IPTCH4C1" and ref["version"] == 1 and ref["nnz"] == len(ri)
    assert ref["counts"] == (8, 8, 4, 4, 70, 1)
    assert ref["norm"] == np.abs(H).sum(axis=1).max()
    np.testing.assert_array_equal(ref["col_ptr"], cp)
    np.testing.assert_array_equal(ref["row_ind"], ri)
    np.testing.assert_array_equal(ref["values"], va)
    np.testing.assert_array_equal(ref["diag"], dg)
    assert not (tmp_path / "gen.bin.tmp").exists()
    # and back through the reader, into the plain path's preparation
    rcp, rri, rva, rdg, _ = api.read_csc_cache(str(path))
    prep = api.prepare_csc(rcp, rri, rva, 70, 3, lift=False)
    np.testing.assert_array_equal(np.sort(prep["diag"]), np.sort(dg))


@pytest.mark.parametrize("defect", ["magic", "version", "short", "col_ptr", "row", "norm_neg",
                                    "norm_nan", "empty"])
def test_rejects_broken_files(lib, golden, tmp_path, defect):
    cp, ri, va = h2o(golden)
    cp, ri = np.array(cp), np.array(ri)
    dg = diag_of(cp, ri, va)
    magic, version, norm = b"IPTH2OC1", 1, 3.0
    if defect == "magic":
        magic = b"XPTH2OC1"
    elif defect == "version":
        version = 2
    elif defect == "col_ptr":
        cp[0] = 1
    elif defect == "row":
        ri[3] = len(cp) + 5
    elif defect == "norm_neg":
        norm = -1.0
    elif defect == "norm_nan":
        norm = float("nan")
    data = oracle.reference_csc_cache_bytes(magic, cp, ri, va, dg, norm, version=version)
    if defect == "short":
        data = data[:-9]
    if defect == "empty":
        data = b""
    path = tmp_path / "bad.bin"
    path.write_bytes(data)
    with pytest.raises(Exception):
        api.read_csc_cache(str(path))


def test_missing_file_and_bad_write_arguments(lib, tmp_path):
    with pytest.raises(Exception):
        api.read_csc_cache(str(tmp_path / "nope.bin"))
    cp = np.array([0, 1, 2], np.int32)
    ri = np.array([0, 1], np.int32)
    with pytest.raises(Exception):
        api.write_csc_cache(str(tmp_path / "x.bin"), cp, ri, [1.0, 2.0], [1.0, 2.0],
                            magic="NOTMAGIC")
    with pytest.raises(Exception):
        api.write_csc_cache(str(tmp_path / "x.bin"), np.array([0, 1, 3], np.int32), ri,
                            [1.0, 2.0], [1.0, 2.0])
