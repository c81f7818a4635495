// Host-only checks of the OBJ reader and the CSV helpers of cpm_ibc.hpp: reads
// the OBJ file argv[1], writes its vertex coordinates to argv[2] (CSV, one row
// per vertex) and a vector to argv[3], reads both back and prints a summary.
#include <cstdio>

#include "cpm_ibc.hpp"

using namespace cpm_gb300;

int main(int argc, char **argv) {
    if (argc < 4) return 2;
    SimplePolygonMesh mesh(argv[1]);
    Helpers::WriteCSV(mesh.vertices, argv[2]);
    std::vector<std::vector<Scalar>> back;
    Helpers::ReadCSV(argv[2], back);
    VectorX v = {0.5, -1.25, 3.0};
    Helpers::WriteCSV(v, argv[3]);
    VectorX w;
    Helpers::ReadCSV(argv[3], w);
    const SurfaceSpecifier s = SurfaceSpecifier::FromMesh(mesh);
    std::printf("vertices %zu faces %zu face0 %zu %zu %zu csv_rows %zu vec %g %g %g kind %d nprims %lld\n", mesh.nVertices(),
                mesh.nFaces(), mesh.faces[0][0], mesh.faces[0][1], mesh.faces[0].size() > 2 ? mesh.faces[0][2] : 0,
                back.size(), w[0], w[1], w[2], s.desc().kind, (long long)s.desc().nprims);
    return 0;
}
