"""container::import (src/container.cc:333-376): the Python mirror reads the
same "id x y z [r]" token stream the reference's fscanf loop reads, and
rejects incomplete or malformed entries.  CPU only (staging, no compute)."""
import io

import numpy as np
import pytest

import voro_gb300 as vg


def _staged(con):
    con._flush_pending()
    return con


def test_import_reads_token_groups_across_lines(tmp_path, monkeypatch):
    got = []
    monkeypatch.setattr(vg._ContainerBase, "put_array", lambda self, ids, xyz, r=None: got.append((ids, xyz, r)))
    con = vg.container.__new__(vg.container)
    con.kind = vg.KIND_CONTAINER
    p = tmp_path / "pts.txt"
    p.write_text("1 0.5 0.25 0.125\n2 0.1\n 0.2 0.3\n\n3 1e-3 2E-2 0.5")
    con.import_file(str(p))
    ids, xyz, r = got[0]
    assert ids.tolist() == [1, 2, 3]
    assert np.array_equal(xyz, [[0.5, 0.25, 0.125], [0.1, 0.2, 0.3], [1e-3, 2e-2, 0.5]])
    assert r is None


def test_import_radical_reads_five_numbers(monkeypatch):
    got = []
    monkeypatch.setattr(vg._ContainerBase, "put_array", lambda self, ids, xyz, r=None: got.append((ids, xyz, r)))
    con = vg.container_poly.__new__(vg.container_poly)
    con.kind = vg.KIND_CONTAINER_POLY
    con.import_file(io.StringIO("7 1 2 3 0.5\n8 4 5 6 0.25\n"))
    ids, xyz, r = got[0]
    assert ids.tolist() == [7, 8] and r.tolist() == [0.5, 0.25]


@pytest.mark.parametrize("text", ["1 0.5 0.5", "1 0.5 0.5 0.5 2", "1 a 0.5 0.5"])
def test_import_error_on_incomplete_or_malformed_entry(text):
    con = vg.container.__new__(vg.container)
    con.kind = vg.KIND_CONTAINER
    with pytest.raises(vg.VoroError):
        con.import_file(io.StringIO(text))
