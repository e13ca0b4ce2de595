"""Writes omega_h_gb300/csrc/ohg_swap3d_tables.inc from the swap3d tables the
reference build dumped into tests/golden/box8_iso.npz.

The edge-swap triangulation tables (all triangulations of the 3..7-gon, their
unique triangles and unique interior edges) define the numbering of the
reference's swap "config" output, so they are kept identical; this file only
re-lays them out as one flat int array:

  per loop size n = 3..7:
    n, nmesh, ntri, nuniq_tri, tri[nuniq_tri][3], mesh_tris[nmesh][ntri],
    nedge, nuniq_edge, edge[nuniq_edge][2], mesh_edges[nmesh][nedge]
"""
import os
import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
t = np.load(os.path.join(ROOT, "tests/golden/box8_iso.npz"))["swap3d_tables"]
out = os.path.join(ROOT, "omega_h_gb300/csrc/ohg_swap3d_tables.inc")
with open(out, "w") as f:
    f.write("// Generated by oracle/gen_swap3d_tables.py: edge-swap triangulation\n")
    f.write("// tables of the 3..7-gon (layout documented there).\n")
    f.write(f"#define OHG_SWAP3D_TABLE_LEN {t.size}\n")
    f.write("OHG_SWAP3D_TABLE_QUAL int const OHG_SWAP3D_TABLE[OHG_SWAP3D_TABLE_LEN] = {\n")
    for i in range(0, t.size, 20):
        f.write("  " + ", ".join(str(int(x)) for x in t[i:i + 20]) + ",\n")
    f.write("};\n")
print(out, t.size)
