"""Host-side logic of the C ABI, on the CPU: exports, option parsing, batch
packing, lookup tables and six-frame translation against the oracle.  No
kernel is launched here."""
import ctypes as C
import json
import re
from pathlib import Path

import numpy as np
import pytest

import hblast
from hblast import synth
from oracle import oracle

ROOT = Path(__file__).resolve().parent.parent
GOLD = json.loads((Path(__file__).parent / "golden" / "reference_tables.json").read_text())


def declared_symbols():
    text = (ROOT / "include" / "hblast_gpu.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(hbg_\w+)\(", text, re.M)))


def test_library_exports_every_declared_symbol(built):
    syms = declared_symbols()
    assert len(syms) >= 20
    L = C.CDLL(str(hblast.library_path()))
    for s in syms:
        assert hasattr(L, s), s
    assert set(syms) <= set(hblast.core._SIGS), set(syms) - set(hblast.core._SIGS)


def test_runtime_options_reference_file(built, tmp_path):
    f = tmp_path / "H-BLAST_runtime_options"
    f.write_text(GOLD["runtime_options_file"])
    o = hblast.read_runtime_options(str(f))
    assert (o.gpu_db_used_ratio, o.fixed_ratio, o.ccr, o.avg_hsps_per_sequence, o.mem_ecc,
            o.balancer_method, o.load_factor, o.chunk_size, o.base_value) == (1.0, 0, 12.0, 20, 0, 1, 4, 200, 100)


def test_runtime_options_fixups_and_missing(built, tmp_path):
    f = tmp_path / "opts"
    f.write_text("#r\n7\n#f\n1\n#ccr\n-3\n#avg\n0\n#ecc\n5\n#bal\n0\n#lf\n-1\n#chunk\n-2\n#base\n-9\n")
    o = hblast.read_runtime_options(str(f))
    assert (o.gpu_db_used_ratio, o.fixed_ratio, o.ccr, o.avg_hsps_per_sequence, o.mem_ecc,
            o.balancer_method, o.load_factor, o.chunk_size, o.base_value) == (0.0, 1, 12.0, 20, 1, 0, 4, 200, 100)
    d = hblast.read_runtime_options(str(tmp_path / "absent"))
    assert d.avg_hsps_per_sequence == 20 and d.load_factor == 4


def test_default_gpu_options(built):
    o = hblast.default_options()
    assert (o.use_gpu, o.num_blocksx, o.num_threadsx, o.method) == (1, 0, 256, 0)


def lut_of_group(batch, g):
    cells, ent, fq, starts = batch.lookup_table(g)
    return cells.astype(np.int64), ent.astype(np.int64), fq, starts


@pytest.mark.parametrize("qlen", [3, 17, 300, 1500])
def test_lookup_table_matches_oracle(built, qlen):
    rng = np.random.default_rng(qlen)
    q = synth.random_letters(rng, qlen)
    b = hblast.Batch.proteins([hblast.ProteinQuery.blastp(q)])
    cells, ent, _, _ = lut_of_group(b, 0)
    cs, oe = oracle.lookup_table(oracle.Query.blastp(q), 11)
    assert np.array_equal(cells, cs) and np.array_equal(ent, oe)


def test_lookup_table_rare_letters(built):
    # every NCBIstdaa letter 1..27 in the query (B, Z, X, U, *, O, J included)
    q = np.array(list(range(1, 28)) * 3, dtype=np.uint8)
    b = hblast.Batch.proteins([hblast.ProteinQuery.blastp(q)])
    cells, ent, _, _ = lut_of_group(b, 0)
    cs, oe = oracle.lookup_table(oracle.Query.blastp(q), 11)
    assert np.array_equal(cells, cs) and np.array_equal(ent, oe)


def test_group_packing_and_offsets(built):
    rng = np.random.default_rng(1)
    qs = [synth.random_letters(rng, n) for n in (100, 900, 800, 50, 9000, 20)]
    b = hblast.Batch.proteins([hblast.ProteinQuery.blastp(x) for x in qs])
    info = b.info()
    assert info["n_queries"] == 6
    # 100+40+900+40+800+40+50 = 1970 <= 2008 share a group; 9000 needs its own
    # (a 16384-entry table in global memory); 20 cannot join it
    assert info["n_groups"] == 3
    seen = 0
    for g in range(info["n_groups"]):
        cells, ent, fq, starts = lut_of_group(b, g)
        # the group's table is the union of its queries' tables, shifted
        for k, st in enumerate(starts):
            cs, oe = oracle.lookup_table(oracle.Query.blastp(qs[fq + k]), 11)
            got = [ent[cells[w]:cells[w + 1]] for w in range(32768)]
            for w in rng.integers(0, 32768, size=500):
                mine = got[w][(got[w] >= st) & (got[w] < st + len(qs[fq + k]))] - st
                assert np.array_equal(mine, oe[cs[w]:cs[w + 1]])
            seen += 1
        if len(starts) > 1:
            assert starts[1] - starts[0] == len(qs[fq]) + 40   # window-sized gap
    assert seen == 6


def test_plain_form_one_query_per_group(built):
    rng = np.random.default_rng(2)
    qs = [synth.random_letters(rng, 60) for _ in range(5)]
    b = hblast.Batch.proteins([hblast.ProteinQuery.blastp(x) for x in qs], max_group_len=1)
    assert b.info()["n_groups"] == 5


def test_blastx_translation_matches_oracle(built):
    rng = np.random.default_rng(4)
    nts = [rng.integers(0, 4, size=n).astype(np.uint8) for n in (300, 301, 302, 1000)]
    nts[1][5] = 9   # an ambiguous base translates to X
    xd = np.full((4, 6), 16, dtype=np.int32)
    cu = np.full((4, 6), 41, dtype=np.int32)
    b = hblast.Batch.blastx(nts, xd, cu, max_group_len=1)
    for k, nt in enumerate(nts):
        prot, off, ln = oracle.translate6(nt)
        cs, oe = oracle.lookup_table(oracle.Query(prot, off, ln, [16] * 6, [41] * 6), 11)
        cells, ent, _, _ = lut_of_group(b, k)
        assert np.array_equal(cells, cs) and np.array_equal(ent, oe)


def smallbone_from_csr(cs, ent):
    """NCBI AaLookupSmallboneCell layout: int32 num_used + union{uint16[3]; int32 cursor}."""
    dt = np.dtype([("num_used", np.int32), ("e", np.uint16, 3), ("pad", np.uint16)])
    cells = np.zeros(32768, dtype=dt)
    overflow = []
    for w in range(32768):
        v = list(ent[cs[w]:cs[w + 1]])[::-1]     # reversed: the library sorts cells
        cells[w]["num_used"] = len(v)
        if len(v) <= 3:
            cells[w]["e"][:len(v)] = v
        else:
            cur = len(overflow)
            overflow += v
            raw = np.array([cur], dtype=np.int32).view(np.uint16)
            cells[w]["e"][0], cells[w]["e"][1] = raw[0], raw[1]
    return cells, np.array(overflow or [0], dtype=np.uint16)


def test_smallbone_import(built):
    rng = np.random.default_rng(6)
    q = synth.random_letters(rng, 250)
    cs, oe = oracle.lookup_table(oracle.Query.blastp(q), 11)
    cells, overflow = smallbone_from_csr(cs, oe)
    assert cells.dtype.itemsize == 12
    b = hblast.Batch.from_smallbone(hblast.ProteinQuery.blastp(q), cells, overflow)
    got_cells, got_ent, _, _ = lut_of_group(b, 0)
    assert np.array_equal(got_cells, cs) and np.array_equal(got_ent, oe)


def test_invalid_inputs_rejected(built):
    bad = np.array([1, 2, 0, 4], dtype=np.uint8)            # sentinel inside a context
    with pytest.raises(hblast.HblastError) as e:
        hblast.Batch.proteins([hblast.ProteinQuery.blastp(bad)])
    assert e.value.code == hblast.core.HBG_ERR_INVALID
    with pytest.raises(hblast.HblastError) as e:
        hblast.Batch.proteins([hblast.ProteinQuery.blastp(np.ones(70000, np.uint8))])
    assert e.value.code == hblast.core.HBG_ERR_TOO_LONG
    with pytest.raises(hblast.HblastError):
        hblast.Batch.proteins([hblast.ProteinQuery.blastp(np.array([1, 2, 30], np.uint8))])


def test_no_device_fails_loudly(built):
    if hblast.device_count() > 0:
        pytest.skip("a GPU is present")
    with pytest.raises(hblast.HblastError) as e:
        hblast.Database(np.ones(10, np.uint8), np.array([0, 10]))
    assert e.value.code == hblast.core.HBG_ERR_NO_DEVICE


def test_tuning_calls_validate_before_upload(built):
    """hbg_batch_tune / hbg_batch_set_mode: argument checks and the host-side
    placement change (no device needed: batches upload at their first search)."""
    rng = np.random.default_rng(7)
    qs = [synth.random_letters(rng, n) for n in (300, 1500)]
    b = hblast.Batch.proteins([hblast.ProteinQuery.blastp(x) for x in qs], max_group_len=2008)
    for bad in ((5, 0), (5000, 0), (-1, 0), (0, 2)):
        with pytest.raises(hblast.HblastError):
            b.tune(*bad)
    b.tune(64, True).tune(0, False)        # valid values; global tables stay chosen
    with pytest.raises(hblast.HblastError):
        b.set_mode(2)
    b.set_mode(1).set_mode(0, 0)
    b.close()


def test_autotune_table_round_trip(tmp_path):
    from hblast import autotune
    rows = [autotune.BucketResult(0, 300, 2, autotune.Choice(4056, 0, 256, 32, True), [])]
    autotune.save(rows, tmp_path / "t.json")
    back = autotune.load(tmp_path / "t.json")
    assert back[0].best == rows[0].best
    assert autotune.choice_for(100, back) == rows[0].best
    assert autotune.choice_for(5000, back) == autotune.Choice(0, 0, 256)


def test_allocation_failure_hook_validates(built):
    """The out-of-memory test hook takes a count and is switched off with 0
    (no device needed)."""
    with pytest.raises(hblast.HblastError):
        hblast.fail_allocations(-1)
    hblast.fail_allocations(2)
    hblast.fail_allocations(0)


def test_schedule_validates_before_upload(built):
    b = hblast.Batch.proteins([hblast.ProteinQuery.blastp(np.ones(50, np.uint8) * 3)])
    b.schedule(4, 8192).schedule(1, 0)
    for bad in ((0, 0), (9, 0), (2, 512), (2, -1)):
        with pytest.raises(hblast.HblastError):
            b.schedule(*bad)
    b.close()
