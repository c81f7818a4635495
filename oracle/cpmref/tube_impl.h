// ORACLE — test infrastructure only. Template part of the Tube restatement.
#pragma once

#include <cmath>
#include <stdexcept>

namespace cpmref {

template <class CPF>
void Tube::BuildWith(const SurfaceSpec &spec, size_t interp_deg, double dx, CPF cpf) {
    Setup(spec, interp_deg, dx);
    BuildTube(cpf);
}

// Tube::BuildTube, dense branch (src/Tube.cpp:295-320, 429-461) with
// FindStartingPoint (:540-551) and AddTubeNode (:554-605).
// Queue order: pop front, then +x,-x,+y,-y,+z,-z; a grid node is marked
// visited (-2) on first sight and kept iff |dist| <= tube radius.
template <class CPF>
void Tube::BuildTube(CPF cpf) {
    const Grid &g = m_grid;
    m_num = 0;
    m_visited = 0;
    m_x.clear();
    m_cpx.clear();
    m_dist.clear();
    m_bdy.clear();
    m_rec.clear();

    // FindStartingPoint: cp of the xstart corner, nearest grid triplet by round().
    V3 corner{g.xstart, g.xstart, g.xstart};
    V3 cp0;
    double d0;
    size_t b0;
    m_surface.ClosestPoint(corner, cp0, d0, b0);
    size_t idx[3];
    for (int d = 0; d < 3; ++d) idx[d] = (size_t)std::round((cp0[d] - g.xstart) / g.dx);
    size_t index = g.Linear(idx[0], idx[1], idx[2]);

    m_map.assign(g.N, -1);
    auto add = [&](size_t rec, const V3 &x, const V3 &cp, double dist, size_t bdy) {
        m_map[rec] = (int64_t)m_num;
        m_rec.push_back(rec);
        m_x.push_back(x);
        m_cpx.push_back(cp);
        m_dist.push_back(dist);
        m_bdy.push_back(bdy);
        m_num++;
    };

    V3 x{g.Coord(idx[0]), g.Coord(idx[1]), g.Coord(idx[2])};
    V3 cp;
    double dist;
    size_t bdy;
    cpf(index, x, cp, dist, bdy);
    m_visited++;
    add(index, x, cp, dist, bdy);  // the seed is added without the band test (src/Tube.cpp:323-327)

    std::vector<size_t> queue;
    queue.reserve(1 << 16);
    queue.push_back(index);
    size_t head = 0;
    while (head < queue.size()) {
        size_t cur = queue[head];
        size_t t[3];
        g.Triplet(cur, t);
        for (int sd = 0; sd < 3; ++sd) {
            for (int sh : {1, -1}) {
                size_t nt[3] = {t[0], t[1], t[2]};
                nt[sd] += (size_t)(ptrdiff_t)sh;
                size_t nbr = g.Linear(nt[0], nt[1], nt[2]);
                if (m_map[nbr] == -1) {
                    m_map[nbr] = -2;
                    V3 xn{g.Coord(nt[0]), g.Coord(nt[1]), g.Coord(nt[2])};
                    cpf(nbr, xn, cp, dist, bdy);
                    m_visited++;
                    if (std::abs(dist) <= m_radius) {
                        queue.push_back(nbr);
                        add(nbr, xn, cp, dist, bdy);
                    }
                }
            }
        }
        head++;
    }

    SetNeighbours();
    m_bpt = ComputeBasePoints(m_cpx);
}

}  // namespace cpmref
