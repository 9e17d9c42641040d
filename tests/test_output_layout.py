"""The output layout (`thermal_init/*`, `obs/configurations`) of a GPU run:
written by dqmc_gb300.output, read back with the HDF5/JLD reader of
tests/golden, and compared with the encodings of the reference's own JLD file
test/data/O3.jld (user block, superblock fields, datatype messages, the
`_creator` group), pinned in the golden fixture."""
import os
import sys

import numpy as np
import pytest

from dqmc_gb300 import output

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import jld_reader  # noqa: E402


@pytest.fixture()
def written(tmp_path):
    rng = np.random.default_rng(5)
    N, M = 16, 10
    conf = rng.uniform(-1, 1, size=(3, N, M))
    confs = [rng.uniform(-1, 1, size=(3, N, M)) for _ in range(7)]
    path = str(tmp_path / "run.out.h5.running")
    jf = output.JLDFile(path)
    output.write_thermal(jf, conf, 250, box=0.2)
    cw = output.ConfigurationWriter(jf, alloc=3)
    for c in confs:
        cw.push(c)
    cw.flush()
    return path, conf, confs


def test_round_trip(written):
    path, conf, confs = written
    t = jld_reader.load_tree(path)
    assert np.array_equal(t["thermal_init/conf"], conf)            # Julia (3, N, M) order
    assert int(t["thermal_init/prethermalized"]) == 250
    assert float(t["thermal_init/box"]) == 0.2
    g = "obs/configurations/"
    assert int(t[g + "count"]) == 7
    assert int(t[g + "alloc"]) == 3
    assert int(t[g + "timeseries/chunk_count"]) == 3
    assert list(t[g + "elsize"]) == [3, 16, 10]
    assert t[g + "eltype"] == "Array{Float64,3}"
    assert t[g + "name"] == "configurations"
    chunks = [t[g + f"timeseries/ts_chunk{i}"] for i in (1, 2, 3)]
    assert [c.shape for c in chunks] == [(3, 16, 10, 3), (3, 16, 10, 3), (3, 16, 10, 1)]
    ts = np.concatenate(chunks, axis=-1)
    for k, c in enumerate(confs):
        assert np.array_equal(ts[..., k], c)


def test_matches_reference_encodings(written, golden):
    path, _, _ = written
    d = open(path, "rb").read()
    assert np.array_equal(np.frombuffer(d[:512], dtype=np.uint8), golden["jld_userblock"])
    r = jld_reader._Reader(path)
    assert r.base == 512
    assert np.array_equal(np.frombuffer(d[512:536], dtype=np.uint8), golden["jld_superblock_head"])
    root = r.links(r.root)
    assert sorted(r.links(root["_creator"])) == list(golden["jld_creator_names"])

    def dtype_msg(addr):
        for mtype, _, data in r.messages(addr):
            if mtype == 0x03:
                return np.frombuffer(bytes(data), dtype=np.uint8)

    ti = r.links(root["thermal_init"])
    want = golden["jld_dt_float64_array"]
    got = dtype_msg(ti["conf"])
    assert np.array_equal(got[:20], want[:20])          # the 20 bytes of the message (rest is padding)
    want = golden["jld_dt_int64_scalar"]
    assert np.array_equal(dtype_msg(ti["prethermalized"])[:12], want[:12])
    cr = r.links(root["_creator"])
    for name in ("JULIA_MAJOR", "JULIA_MINOR", "JULIA_PATCH", "ENDIAN_BOM"):
        assert np.array_equal(dtype_msg(cr[name])[:12], golden["jld_dt_uint32_scalar"][:12])
    assert np.array_equal(dtype_msg(cr["WORD_SIZE"])[:12], golden["jld_dt_int64_scalar"][:12])
    eof = np.frombuffer(d[512 + 40:512 + 48], dtype="<u8")[0]
    assert eof == len(d)


def test_rewrite_keeps_earlier_chunks(tmp_path):
    """A second thermal save and further pushes rewrite the file with every
    earlier dataset still present (the reference deletes and rewrites
    thermal_init on each save, src/dqmc_framework.jl:322-333)."""
    path = str(tmp_path / "x.jld")
    jf = output.JLDFile(path)
    cw = output.ConfigurationWriter(jf, alloc=2)
    for k in range(4):
        cw.push(np.full((3, 4, 2), float(k)))
        output.write_thermal(jf, np.full((3, 4, 2), 10.0 + k), k + 1)
    t = jld_reader.load_tree(path)
    assert int(t["thermal_init/prethermalized"]) == 4
    assert np.all(t["thermal_init/conf"] == 13.0)
    assert int(t["obs/configurations/count"]) == 4
    assert np.array_equal(t["obs/configurations/timeseries/ts_chunk2"][0, 0, 0], [2.0, 3.0])
