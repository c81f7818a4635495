"""Input formats (host code, no GPU): the OBJ reader and CSV helpers of the C++
header (SimplePolygonMesh::readMeshFromFile, Helpers::WriteCSV/ReadCSV), and the
Python reader, on small files written here."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

OBJ = """# a tetrahedron, one face continued over two lines, normals and uv ignored
v 0 0 0
v 1 0 0
v 0 1 0
v 0 0 1
vt 0 0
vn 0 0 1
f 1/1/1 3/1/1 2/1/1
f 1//1 2//1 4//1
f 1 4 \\
  3
f 2 3 4
"""

POLY = """v 1 0 0
v 0 1 0
v -1 0 0
l 1 2 3 1
"""


def test_cpp_obj_and_csv(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    exe = tmp_path / "io_example"
    subprocess.run([gxx, "-std=c++17", "-Wall", "-Werror", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "io_example.cpp"), "-o", str(exe)], check=True)
    (tmp_path / "t.obj").write_text(OBJ)
    out = subprocess.run([str(exe), str(tmp_path / "t.obj"), str(tmp_path / "v.csv"), str(tmp_path / "w.csv")],
                         check=True, capture_output=True, text=True).stdout.split()
    rec = dict(zip(out[0::2], out[1::2]))
    assert rec["vertices"] == "4" and rec["faces"] == "4" and rec["csv_rows"] == "4"
    assert out[out.index("face0") + 1:out.index("face0") + 4] == ["0", "2", "1"]
    assert out[out.index("vec") + 1:out.index("vec") + 4] == ["0.5", "-1.25", "3"]
    assert rec["nprims"] == "4"
    rows = [list(map(float, l.split(","))) for l in (tmp_path / "v.csv").read_text().splitlines()]
    assert rows == [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]]
    (tmp_path / "p.obj").write_text(POLY)
    out = subprocess.run([str(exe), str(tmp_path / "p.obj"), str(tmp_path / "v2.csv"), str(tmp_path / "w2.csv")],
                         check=True, capture_output=True, text=True).stdout.split()
    rec = dict(zip(out[0::2], out[1::2]))
    assert rec["faces"] == "3" and rec["nprims"] == "3"


def test_python_obj_reader(tmp_path):
    from cpm_gb300 import io as cio

    (tmp_path / "t.obj").write_text(OBJ)
    v, f = cio.read_obj(str(tmp_path / "t.obj"))
    assert v.shape == (4, 3) and f.shape == (4, 3)
    assert f[0].tolist() == [0, 2, 1] and f[2].tolist() == [0, 3, 2]
    (tmp_path / "p.obj").write_text(POLY)
    v, f = cio.read_obj(str(tmp_path / "p.obj"))
    assert f.tolist() == [[0, 1], [1, 2], [2, 0]]
    cio.write_csv(str(tmp_path / "a.csv"), np.array([0.5, -1.25, 3.0]))
    assert cio.read_csv(str(tmp_path / "a.csv")).tolist() == [[0.5, -1.25, 3.0]]
