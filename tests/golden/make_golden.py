"""Regenerates the golden fixtures in this directory from the reference itself.

Runs only where the reference sources are present: it builds oracle/_ref/fsm
(the reference's own gspan.cu/graph.cc/fsm.cu with support computed on the
CPU, see oracle/ref_support_shim.h) and records, for each seeded graph of
CASES and each (min_support, k), the pattern lines the reference prints
(its final timing line removed).  Graphs are not stored: they are rebuilt
from gspan_gb300.datagen by the tests, and the sha256 of their binary CSR
file is stored to catch generator drift.

    python tests/golden/make_golden.py

Large cases (``--large``): jobs whose last level the reference would have to
materialise in host memory beyond any test host (the 100,000-vertex Chung-Lu
graph at 3 edges holds about 1.9e10 three-edge embeddings).  Their lines come
from the oracle port with ``--stream-last``: the same rules and support
semantics, the last level counted without storing it.  That mode is checked
against the reference's own output on every small case above
(tests/test_oracle.py) before it is trusted here.  Written to
large_manifest.json with the job's extended-embedding count.

    python tests/golden/make_golden.py --large
"""
import gzip
import hashlib
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from gspan_gb300 import datagen  # noqa: E402

# (name, generator call, [(min_support, k), ...])
CASES = [
    ("er3300", "datagen.er_3300(0)", [(300, 3), (200, 3), (50, 3), (20, 3)]),
    ("er_small_multilabel", "datagen.erdos_renyi(400, 700, 4, 5, nelabels=3)", [(10, 3), (4, 4)]),
    ("cl_2k", "datagen.chung_lu(2000, 6000, 2.1, 6, 1.0, 11, max_deg=120)", [(150, 3), (60, 3)]),
    ("multigraph_loops", "datagen.random_multigraph(30, 80, 3, 2, 21, self_loops=True)", [(1, 3), (2, 4)]),
    ("multigraph_plain", "datagen.random_multigraph(40, 90, 2, 3, 22, self_loops=False)", [(2, 4), (3, 3)]),
    ("star_path", "datagen.csr_from_edge_list(7, [0,1,1,1,0,2,1], [0,0,0,1,2,3], [1,2,3,4,5,6], [0,0,1,0,1,0])",
     [(1, 4), (1, 1)]),
    ("triangle_4cycle", "datagen.csr_from_edge_list(7, [0,0,0,1,1,1,1], [0,1,2,3,4,5,6], [1,2,0,4,5,6,3], [0]*7)",
     [(1, 3), (2, 4)]),
    ("empty", "datagen.csr_from_edge_list(0, [], [], [], [])", [(1, 3)]),
    ("isolated", "datagen.csr_from_edge_list(5, [3,1,4,1,5], [], [], [])", [(1, 3)]),
    ("negative_labels", "datagen.csr_from_edge_list(6, [-5,7,-5,100,7,-5], [0,1,2,3,4,5], [1,2,3,4,5,0], [-2,9,-2,9,-2,9])",
     [(1, 4)]),
]


# (name, generator call, min_support, k)
LARGE_CASES = [
    ("chung_lu_100k", "datagen.chung_lu_100k(1)", 10000, 3),
    # The 3.7M-vertex configuration (exponent 2.3, degree cap sqrt(2m), 37
    # labels Zipf(0.8), seed 3) scaled to 20,000 vertices with the same mean
    # degree, min support scaled likewise (20,000 x 20,000 / 3.7M), 4 edges.
    ("chung_lu_3_7m_scaled_20k", "datagen.chung_lu(20000, 89189, 2.3, 37, 0.8, 3, max_deg=(2 * 89189) ** 0.5)",
     108, 4),
]


def make_large() -> None:
    port = os.path.join(ROOT, "oracle", "_port", "fsm_port")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    manifest = []
    with tempfile.TemporaryDirectory() as tmp:
        for name, expr, sup, k in LARGE_CASES:
            g = eval(expr, {"datagen": datagen})
            path = os.path.join(tmp, name + ".bin")
            g.save(path)
            r = subprocess.run([port, path, str(sup), str(k), "--stats", "--stream-last"], capture_output=True,
                               text=True, check=True)
            out = r.stdout.splitlines()
            assert out and out[-1].startswith("load:"), out[-1:]
            st = json.loads(r.stderr.strip().splitlines()[-1])
            body = "".join(line + "\n" for line in out[:-1]).encode()
            fname = f"{name}_s{sup}_k{k}.txt"
            if len(body) > 64 << 10:   # long outputs are stored gzipped (fixed mtime: reproducible bytes)
                fname += ".gz"
                with open(os.path.join(HERE, fname), "wb") as raw:
                    with gzip.GzipFile(fileobj=raw, mode="wb", mtime=0) as f:
                        f.write(body)
            else:
                with open(os.path.join(HERE, fname), "wb") as f:
                    f.write(body)
            manifest.append({"name": name, "graph": expr, "sha256": hashlib.sha256(g.to_bytes()).hexdigest(),
                             "min_support": sup, "k": k, "expected": fname, "patterns": len(out) - 1,
                             "seeds": st["seeds"], "extended": st["extended"],
                             "source": "oracle port, --stream-last"})
    with open(os.path.join(HERE, "large_manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)
        f.write("\n")


def main() -> None:
    ref = os.path.join(ROOT, "oracle", "_ref", "fsm")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    manifest = []
    with tempfile.TemporaryDirectory() as tmp:
        for name, expr, runs in CASES:
            g = eval(expr, {"datagen": datagen})
            path = os.path.join(tmp, name + ".bin")
            g.save(path)
            digest = hashlib.sha256(g.to_bytes()).hexdigest()
            for sup, k in runs:
                out = subprocess.run([ref, path, str(sup), str(k)], capture_output=True, text=True, check=True,
                                     env={**os.environ, "OMP_NUM_THREADS": "4"}).stdout.splitlines()
                assert out and out[-1].startswith("load:"), out[-1:]
                fname = f"{name}_s{sup}_k{k}.txt"
                with open(os.path.join(HERE, fname), "w") as f:
                    f.write("".join(line + "\n" for line in out[:-1]))
                manifest.append({"name": name, "graph": expr, "sha256": digest, "min_support": sup, "k": k,
                                 "expected": fname, "patterns": len(out) - 1})
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    if "--large" in sys.argv[1:]:
        make_large()
    else:
        main()
