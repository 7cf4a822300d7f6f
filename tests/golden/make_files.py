"""Writes the hand-made STP cases of this folder (deterministic formulas, no randomness).

  path3000.stp  a path of 3000 vertices plus a few long chords: relaxation
                needs many frontier sweeps
  star129.stp   a star: every shortest path passes the centre
  dup5.stp      a terminal listed twice
  dense40.stp   the complete graph on 40 vertices
"""
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def write(name, n, edges, terms, cost=None):
    lines = ["33d32945 stp file, stp format version 1.0", "", "section comment", f'name    "{name}"',
             'creator "emv-gb300 tests"', "end", "", "section graph", f"nodes {n}", f"edges {len(edges)}"]
    lines += [f"e {u} {v} {w}" for u, v, w in edges]
    lines += ["end", "", "section terminals", f"terminals {len(terms)}"] + [f"t {t}" for t in terms] + ["end", ""]
    if cost is not None:
        lines.append(f"cost {cost}")
    lines.append("eof")
    with open(os.path.join(HERE, name), "w") as f:
        f.write("\n".join(lines) + "\n")


# 1-based vertex ids in the files
path = [(i, i + 1, 1 + (i * 7919) % 97) for i in range(1, 3000)]
path += [(1 + (j * 613) % 3000, 1 + (j * 1543 + 11) % 3000, 500 + j) for j in range(1, 9)]
write("path3000.stp", 3000, path, [1, 3000, 1500, 750, 2250])

star = [(1, i, 1 + (i * 37) % 23) for i in range(2, 130)]
write("star129.stp", 129, star, [2, 40, 77, 101, 128, 129])

dup = [(i, i % 60 + 1, 1 + (i * 13) % 17) for i in range(1, 61)] + [(i, (i * 7) % 60 + 1, 5 + i % 9)
                                                                     for i in range(1, 61)]
write("dup5.stp", 60, dup, [3, 17, 3, 44, 59])

dense = [(u, v, 1 + (u * 31 + v * 17) % 50) for u in range(1, 41) for v in range(u + 1, 41)]
write("dense40.stp", 40, dense, [1, 5, 9, 13, 22, 30, 35, 40])
