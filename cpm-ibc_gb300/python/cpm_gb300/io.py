"""Input formats: OBJ meshes and polylines (SimplePolygonMesh::readMeshFromObjFile,
src/SimplePolygonMesh.cpp:138-222) and comma-separated values (Helpers::WriteCSV /
ReadCSV, src/Helpers.cpp:11-82)."""
import numpy as np


def read_obj(path):
    """(vertices [n, 3], faces [m, k]) of an OBJ file: "v" records, "f" faces of
    "v", "v/vt", "v//vn" or "v/vt/vn" tokens (1-based; a "\\" token continues the
    face on the next line), "l" polylines as consecutive segments (k = 2)."""
    verts, faces = [], []
    with open(path) as f:
        lines = iter(f.read().splitlines())
        for line in lines:
            tok = line.split()
            if not tok:
                continue
            if tok[0] == "v":
                verts.append([float(t) for t in tok[1:]])
            elif tok[0] == "f":
                face, rest = [], tok[1:]
                while rest:
                    t = rest.pop(0)
                    if t == "\\":
                        rest = next(lines, "").split()
                        continue
                    face.append(int(t.split("/")[0]) - 1)
                faces.append(face)
            elif tok[0] == "l":
                ids = [int(t) - 1 for t in tok[1:]]
                faces.extend([ids[i], ids[i + 1]] for i in range(len(ids) - 1))
    return np.array(verts, np.float64), np.array(faces, np.int64)


def write_csv(path, data):
    """one line per row (a vector is one line)"""
    rows = np.atleast_2d(np.asarray(data))
    with open(path, "w") as f:
        for r in rows:
            f.write(",".join(repr(float(v)) for v in r) + "\n")


def read_csv(path):
    with open(path) as f:
        return np.array([[float(t) for t in line.split(",")] for line in f.read().splitlines() if line.strip()])
