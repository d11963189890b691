"""Input formats: the seeded generators, the reference's text and binary CSR
formats, and this library's drop-in `convert` (graph.h loader on the CPU)."""
import hashlib
import os
import subprocess

import numpy as np
import pytest

from helpers import ROOT, golden_cases
from gspan_gb300 import datagen

CONVERT = os.path.join(ROOT, "gspan_gb300", "_lib", "convert")
REF_CONVERT = os.path.join(ROOT, "oracle", "_ref", "convert")


def test_generators_are_deterministic():
    case = [c for c in golden_cases() if c["name"] == "er3300"][0]
    a = datagen.er_3300(0)
    b = datagen.er_3300(0)
    assert a.to_bytes() == b.to_bytes()
    assert hashlib.sha256(a.to_bytes()).hexdigest() == case["sha256"]


def test_er_3300_shape():
    g = datagen.er_3300(0)
    assert g.n == 3300 and g.m == 2 * 4700
    assert not (g.edges[:, 0] == g.edges[:, 1]).any()
    assert set(np.unique(g.vlabels)) == set(range(6))


def test_chung_lu_100k_shape():
    g = datagen.chung_lu_100k(1)
    deg = np.diff(g.offsets)
    assert g.n == 100_000 and g.m == 2 * 1_080_000
    assert 1200 <= deg.max() <= 1600
    counts = np.bincount(g.vlabels, minlength=29)
    assert counts.shape[0] == 29 and counts[0] > counts[1] > counts[5]


def _csr_invariants(g):
    assert g.offsets[0] == 0 and g.offsets[-1] == g.m
    for v in range(g.n):
        seg = g.edges[g.offsets[v]:g.offsets[v + 1]]
        assert (seg[:, 0] == v).all()
        keys = list(zip(seg[:, 1], seg[:, 2]))
        assert keys == sorted(keys)


@pytest.mark.parametrize("name", ["multigraph_loops", "negative_labels", "star_path", "isolated", "empty"])
def test_convert_matches_numpy_csr(name, tmp_path):
    case = [c for c in golden_cases() if c["name"] == name][0]
    g = eval(case["graph"], {"datagen": datagen})
    _csr_invariants(g)
    txt = tmp_path / "g.txt"
    txt.write_text(datagen.to_gspan_text(g))
    out = tmp_path / "g.bin"
    r = subprocess.run([CONVERT, str(txt), str(out)], capture_output=True, text=True, check=True)
    assert r.stdout.startswith(f"|V| = {g.n} |E| = ")
    assert out.read_bytes() == g.to_bytes()
    if os.path.exists(REF_CONVERT):
        out2 = tmp_path / "ref.bin"
        subprocess.run([REF_CONVERT, str(txt), str(out2)], capture_output=True, check=True)
        assert out2.read_bytes() == out.read_bytes()


def test_text_loader_semantics(tmp_path):
    """`t` lines merge graphs, vertices only named by edges get label 0, ids are
    renumbered in ascending order, adjacency sorted by (to, label)."""
    txt = tmp_path / "g.txt"
    txt.write_text("t # 0\nv 10 5\nv 3 7\ne 10 3 2\nt # 1\ne 3 42 1\ne 10 3 0\n")
    out = tmp_path / "g.bin"
    subprocess.run([CONVERT, str(txt), str(out)], capture_output=True, check=True)
    g = datagen.load_bin(str(out))
    assert g.n == 3 and g.m == 6
    assert list(g.vlabels) == [7, 5, 0]          # ids 3, 10, 42
    assert g.edges[g.offsets[0]:g.offsets[1]].tolist() == [[0, 1, 0], [0, 1, 2], [0, 2, 1]]


def test_truncated_binary_is_rejected(tmp_path):
    g = datagen.er_3300(0)
    path = tmp_path / "t.bin"
    path.write_bytes(g.to_bytes()[:-7])
    with pytest.raises(ValueError):
        datagen.load_bin(str(path))
    r = subprocess.run([os.path.join(ROOT, "gspan_gb300", "_lib", "fsm"), str(path), "10", "2"],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "bad edges" in r.stderr


def test_missing_file_is_rejected():
    r = subprocess.run([os.path.join(ROOT, "gspan_gb300", "_lib", "fsm"), "/nonexistent.bin", "10", "2"],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "failed to open file" in r.stderr


# Malformed records: the reference's reader (graph.cc:38-64) keeps reading; a
# failed conversion leaves that variable and the record's later ones as the
# previous record set them, and the record is still added.
MALFORMED = [
    "v 0 1\nv 1 2\ne 0 1 0\nv x 3\nv 2 5\ne 1 2 0\n",
    "v 1 2\nv 2 2\ne 1 2 0\nv abc 3\ne 1 3 0\nv 3 2\n",
    "v 1 2\nv 2 2\ne 1 2 0\ne 1\n",
    "v 1 2 v 2 2 e 1 2 0 e 2 - 0 e 1 1 0",
    "v 1 2\ne 1 2 0\nv 12ab 3\ne 4 5 7\n",
    "t # 0\nv 1 2\ne 1 2 3\ne 4 x\nv 9\n",
    "t # x\nv 1 2\n",
    "v 1 2\ne 1 2 0\ne 7 -\n",
]


@pytest.mark.parametrize("text", MALFORMED)
def test_convert_reads_malformed_records_like_the_reference(text, tmp_path):
    src = tmp_path / "g.txt"
    src.write_text(text)
    out = tmp_path / "g.bin"
    r = subprocess.run([CONVERT, str(src), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    if os.path.exists(REF_CONVERT):
        ref_out = tmp_path / "ref.bin"
        rr = subprocess.run([REF_CONVERT, str(src), str(ref_out)], capture_output=True, text=True, check=True)
        assert rr.stdout == r.stdout
        assert ref_out.read_bytes() == out.read_bytes()


def test_convert_stale_values_by_hand(tmp_path):
    """'v x 3' fails at its id: the reference still adds vertex v with the values
    the previous record ('e 0 1 0') left, id 1 and label 0, relabelling vertex
    1; 'x' and '3' are then skipped as record heads."""
    src = tmp_path / "g.txt"
    src.write_text("v 0 1\nv 1 2\ne 0 1 0\nv x 3\nv 2 5\ne 1 2 0\n")
    out = tmp_path / "g.bin"
    subprocess.run([CONVERT, str(src), str(out)], capture_output=True, check=True)
    g = datagen.load_bin(str(out))
    assert g.vlabels.tolist() == [1, 0, 5] and g.m == 4


@pytest.mark.parametrize("text", ["v 1\n", "t # 5\ne x\n", "e 1 2\n"])
def test_convert_refuses_values_never_assigned(text, tmp_path):
    """The reference would read an uninitialised variable here (undefined)."""
    src = tmp_path / "g.txt"
    src.write_text(text)
    r = subprocess.run([CONVERT, str(src), str(tmp_path / "g.bin")], capture_output=True, text=True)
    assert r.returncode != 0 and "malformed record" in r.stderr
