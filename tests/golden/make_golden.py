"""Generate tests/golden/reference_loaders.json -- run in the development
container, where the reference checkout and oracle/_ref exist.

For each small MatrixMarket input below, the reference's own host code
(compiled from its sources by oracle/build_ref.sh) loads the file:
  * ref_dump_coo: Graph::ReadGraph + VirtualGraph::MakeUGraph
    (index2core/shared/graph.cpp:17-95, virtual_graph.cpp:12-192), the
    loader of HistoCore / CntCore / NbrCore / peelone / gppeel;
  * ref_dump_csr: Graph::readFile (peel/src/graph.cpp:58-133), the loader of
    peelone_dyn / peel_dyn (1-based inputs only: it shifts every id down by one).
Their arrays are stored verbatim.  Core numbers are added from the oracle's
Batagelj-Zaversnik peel and, where the graph is simple, from networkx as an
independent cross-check.  The `example` case is the reference's own
example.txt, whose known answer is core 2 for all five vertices.

Usage:  python tests/golden/make_golden.py
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402

REF_DIR = os.environ.get("PICO_REFERENCE_DIR", "/root/reference")


def mm_text(edges, n_hint, weights=True, extra_lines=()):
    lines = ["%%MatrixMarket matrix coordinate integer symmetric",
             "%d %d %d" % (n_hint, n_hint, len(edges) + len(extra_lines))]
    for i, (u, v) in enumerate(edges):
        lines.append("%d %d 1" % (u, v) if (weights and i % 3 != 2) else "%d %d" % (u, v))
    lines.extend(extra_lines)
    return "\n".join(lines) + "\n"


def cases():
    rng = np.random.default_rng(20221130)
    out = {}
    with open(os.path.join(REF_DIR, "example.txt")) as f:
        out["example"] = f.read()
    # 0-based ids with duplicates (both orders) and self-loops
    e = [(0, 1), (1, 2), (2, 0), (2, 3), (3, 3), (1, 0), (0, 1), (4, 2), (4, 4), (5, 0)]
    out["zero_based_dups"] = mm_text(e, 6)
    # 1-based, duplicates, self-loops, a weight column on some lines only
    e = [(1, 2), (2, 3), (3, 1), (3, 4), (4, 3), (2, 2), (5, 6), (6, 5), (5, 6), (1, 7), (7, 7), (4, 1)]
    out["dups_selfloops"] = mm_text(e, 7)
    # unused ids inside the range (isolated vertices), max id used once
    e = [(2, 5), (5, 9), (9, 2), (9, 12), (12, 2), (5, 12), (20, 12)]
    out["sparse_ids"] = mm_text(e, 20)
    # a hub of degree 150 (three 64-wide virtual nodes) plus a random tail
    e = [(1, j) for j in range(2, 152)]
    for _ in range(300):
        u, v = rng.integers(2, 152, size=2)
        e.append((int(u), int(v)))
    out["hub150"] = mm_text(e, 151)
    # Erdos-Renyi-like: n=300, 1200 uniform pairs (duplicates possible)
    e = [(int(a) + 1, int(b) + 1) for a, b in rng.integers(0, 300, size=(1200, 2))]
    out["er300"] = mm_text(e, 300)
    # R-MAT-like scale 9, 2048 pairs (skewed; many duplicates)
    pairs = []
    for _ in range(2048):
        u = v = 0
        for bit in range(9):
            r = rng.random()
            if r < 0.57:
                q = 0
            elif r < 0.76:
                q = 1
            elif r < 0.95:
                q = 2
            else:
                q = 3
            u |= (q >> 1) << bit
            v |= (q & 1) << bit
        pairs.append((u + 1, v + 1))
    out["rmat9"] = mm_text(pairs, 512)
    # a deep core: clique on 40 vertices + a path hanging off it
    e = [(i, j) for i in range(1, 41) for j in range(i + 1, 41)]
    e += [(40 + i, 41 + i) for i in range(0, 30)]
    out["clique40_path"] = mm_text(e, 70)
    # degenerate inputs
    out["no_edges"] = mm_text([], 0)
    out["only_selfloops"] = mm_text([(1, 1), (2, 2), (3, 3)], 3)
    return out


def read_coo_dump(path):
    b = open(path, "rb").read()
    hdr = np.frombuffer(b[:16], dtype=np.uint32)
    n, m, has_zero, part = (int(x) for x in hdr)
    num_parts = int(np.frombuffer(b[16:24], dtype=np.uint64)[0])
    a = np.frombuffer(b[24:], dtype=np.uint32)
    o = 0
    edges = a[o:o + 2 * m].reshape(m, 2); o += 2 * m
    outdeg = a[o:o + n]; o += n
    nodeptr = a[o:o + n]; o += n
    edgelist = a[o:o + 2 * m + n]; o += 2 * m + n
    parts = a[o:o + 2 * num_parts].reshape(num_parts, 2); o += 2 * num_parts
    assert o == a.size
    return dict(n=n, m=m, has_zero=bool(has_zero), part_size=part, num_parts=num_parts,
                src=edges[:, 0].tolist(), dst=edges[:, 1].tolist(), out_degree=outdeg.tolist(),
                node_pointer=nodeptr.tolist(), edge_list=edgelist.tolist(), parts=parts.tolist())


def read_csr_dump(path):
    a = np.frombuffer(open(path, "rb").read(), dtype=np.uint32)
    V, E = int(a[0]), int(a[1])
    o = 2
    deg = a[o:o + V]; o += V
    off = a[o:o + V + 1]; o += V + 1
    nb = a[o:o + E]; o += E
    assert o == a.size
    return dict(V=V, E=E, degrees=deg.tolist(), offsets=off.tolist(), neighbors=nb.tolist())


def main():
    ref_coo = os.path.join(ROOT, "oracle", "_ref", "ref_dump_coo")
    ref_csr = os.path.join(ROOT, "oracle", "_ref", "ref_dump_csr")
    if not os.path.exists(ref_coo):
        oracle.build_ref()
    import networkx as nx
    fixtures = {}
    for name, text in cases().items():
        with tempfile.TemporaryDirectory() as td:
            mtx = os.path.join(td, name + ".mtx")
            with open(mtx, "w") as f:
                f.write(text)
            subprocess.check_call([ref_coo, mtx, os.path.join(td, "coo.bin")], stdout=subprocess.DEVNULL)
            coo = read_coo_dump(os.path.join(td, "coo.bin"))
            one_based = not coo["has_zero"]
            csr = None
            if one_based:
                os.makedirs(os.path.join(td, "output"))
                subprocess.check_call([ref_csr, mtx, os.path.join(td, "csr.bin")], cwd=td,
                                      stdout=subprocess.DEVNULL)
                csr = read_csr_dump(os.path.join(td, "csr.bin"))
        n = coo["n"]
        rp, col = oracle.csr_multi(n, coo["src"], coo["dst"])
        core_multi, kmax_multi = oracle.bz(rp, col)
        entry = dict(text=text, coo=coo, core_bz_coo=core_multi.tolist(), kmax_coo=kmax_multi)
        if csr is not None:
            V = csr["V"]
            rpd = np.array(csr["offsets"], dtype=np.int64)
            cd = np.array(csr["neighbors"], dtype=np.uint32)
            core_d, kmax_d = oracle.bz(rpd, cd)
            g = nx.Graph()
            g.add_nodes_from(range(V))
            for v in range(V):
                for u in cd[rpd[v]:rpd[v + 1]]:
                    g.add_edge(v, int(u))
            cn = nx.core_number(g)
            entry.update(csr=csr, core_bz_csr=core_d.tolist(), kmax_csr=kmax_d,
                         core_networkx_csr=[int(cn[v]) for v in range(V)])
        if name == "example":
            entry["known_answer"] = [2, 2, 2, 2, 2]
        fixtures[name] = entry
    out = os.path.join(HERE, "reference_loaders.json")
    with open(out, "w") as f:
        json.dump(fixtures, f, separators=(",", ":"))
    print("wrote", out, os.path.getsize(out), "bytes,", len(fixtures), "cases")


if __name__ == "__main__":
    main()
