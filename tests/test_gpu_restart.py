"""Restart files (ib3d_write_restart / ib3d_read_restart and the reference's text
`result` format): a run written out after some steps and read into a fresh
context continues bit for bit like the uninterrupted run, and the binary file's
layout is the documented one."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_binary_restart_continues_bit_exact(ib3d, grids, tmp_path):
    cs = grids.case("tiny")
    a = ib3d.setup_case(cs)
    for step in range(1, 4):
        a.step(step == 1)
    path = tmp_path / "state.ib3d"
    a.write_restart(path, totime=3 * cs.dt, ita=3, ita1=7)
    # the documented layout: 64-byte header, then u, v, w, p (Fortran order)
    raw = path.read_bytes()
    n3 = int(np.prod(a.shape))
    assert raw[:8] == b"IB3DRST1" and len(raw) == 64 + 4 * 8 * n3
    hdr = np.frombuffer(raw[8:64], dtype="<i8")
    assert tuple(hdr[:3]) == cs.shape and hdr[4] == 3 and hdr[5] == 7 and hdr[6] == 4
    u = np.frombuffer(raw[64:64 + 8 * n3], dtype="<f8").reshape(a.shape, order="F")
    assert np.array_equal(u, a.get_field("u"))
    b = ib3d.setup_case(cs)
    totime, ita, ita1 = b.read_restart(path)
    assert (totime, ita, ita1) == (3 * cs.dt, 3, 7)
    for f in ("u", "v", "w", "p", "ut", "vt", "wt"):
        assert np.array_equal(b.get_field(f), a.get_field(f)), f
    for step in range(2):      # the first step after a restart re-brackets the drag probes (stressCal1)
        sa, ca = a.step(False)
        sb, cb = b.step(step == 0)
        assert sa["sweeps"] == sb["sweeps"] and np.array_equal(ca, cb)
    for f in ("u", "v", "w", "p"):
        assert np.array_equal(b.get_field(f), a.get_field(f)), f
    a.close()
    b.close()


def test_reference_text_result_round_trip(ib3d, grids, tmp_path):
    cs = grids.case("tiny")
    a = ib3d.setup_case(cs)
    a.step(True)
    path = tmp_path / "result"
    a.write_restart(path, totime=0.25, ita=1, ita1=0, text=True)
    lines = path.read_text().splitlines()
    assert len(lines) == int(np.prod(a.shape)) and len(lines[0].split()) == 7
    b = ib3d.setup_case(cs)
    assert b.read_restart(path, text=True) == (0.25, 1, 0)
    for f in ("u", "v", "w", "p"):
        assert np.array_equal(b.get_field(f), a.get_field(f)), f
    # a record written by hand in list-directed style (commas, exponent forms) reads too
    vals = np.loadtxt(path)
    with open(tmp_path / "result2", "w") as fh:
        for row in vals:
            fh.write(", ".join(repr(float(x)) for x in row[:5]) + f", {int(row[5])}, {int(row[6])}\n")
    c = ib3d.setup_case(cs)
    c.read_restart(tmp_path / "result2", text=True)
    assert np.array_equal(c.get_field("p"), a.get_field("p"))
    for s in (a, b, c):
        s.close()


def test_restart_errors(ib3d, grids, tmp_path):
    cs = grids.case("tiny")
    a = ib3d.setup_case(cs)
    with pytest.raises(ib3d.IB3DError) as e:
        a.read_restart(tmp_path / "missing")
    assert e.value.code == ib3d.ERR_IO
    other = ib3d.setup_case(grids.case("small"))
    other.write_restart(tmp_path / "small.ib3d")
    with pytest.raises(ib3d.IB3DError) as e:
        a.read_restart(tmp_path / "small.ib3d")
    assert e.value.code == ib3d.ERR_ARG
    (tmp_path / "short").write_bytes((tmp_path / "small.ib3d").read_bytes()[:1000])
    with pytest.raises(ib3d.IB3DError) as e:
        other.read_restart(tmp_path / "short")
    assert e.value.code == ib3d.ERR_IO
    a.close()
    other.close()


def test_library_result_file_restarts_the_oracle_bit_exact(ib3d, grids, oracle_mod, tmp_path):
    """The library writes the reference's `result` file after 3 steps; the oracle's
    own restatement of lastConditions (subLastConditions.f90:2-42) reads it, and both
    continue for 3 steps: sweep counts, drag/lift and fields must be bit-identical.
    The reverse direction too: the library reads the oracle's writeResult file
    (subWriteOutput.f90:62-72), including records split across lines."""
    cs = grids.case("tiny")
    s = ib3d.setup_case(cs)
    for step in range(1, 4):
        s.step(step == 1)
    path = tmp_path / "result"
    s.write_restart(path, totime=3 * cs.dt, ita=3, ita1=3, text=True)
    o = oracle_mod.setup_case(cs)
    assert o.read_result_text(path) == (3 * cs.dt, 3, 3)
    for f in ("u", "v", "w", "p", "ut", "vt", "wt"):
        assert np.array_equal(o.get_field(f), s.get_field(f)), f
    for step in range(3):   # both re-bracket the drag probes on the first step after the restart
        ss, cs_ = s.step(step == 0)
        so, co = o.step(step == 0)
        assert ss["sweeps"] == so["sweeps"], step
        assert np.array_equal(cs_, co), step
    for f in ("u", "v", "w", "p"):
        assert np.array_equal(o.get_field(f), s.get_field(f)), f
    # the oracle's file, each record broken over two lines, read by the library
    path2 = tmp_path / "result_oracle"
    o.write_result_text(path2, 6 * cs.dt, 6, 6)
    lines = path2.read_text().splitlines()
    split = []
    for ln in lines:
        v = ln.split()
        split += [" ".join(v[:3]), ", ".join(v[3:])]
    path2.write_text("\n".join(split) + "\n")
    b = ib3d.setup_case(cs)
    assert b.read_restart(path2, text=True) == (6 * cs.dt, 6, 6)
    for f in ("u", "v", "w", "p"):
        assert np.array_equal(b.get_field(f), o.get_field(f)), f
    for x in (s, o, b):
        x.close()
