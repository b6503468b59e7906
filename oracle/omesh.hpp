// omesh.hpp -- the oracle's hexahedral block mesh.
//
// TEST INFRASTRUCTURE ONLY: the checker's own statement of the mesh the
// picFoam hot path runs on.  It is written from OpenFOAM's polyMesh
// conventions as picFoam uses them (owner cells, outward face area vectors,
// the face-fan tet decomposition of Macpherson, Nordin & Weller, Commun.
// Numer. Meth. Engng 25 (2009) 263, which picFoam's VolumeWeighting walks in
// PICMCCFVM/submodels/ChargeDistribution/VolumeWeighting/VolumeWeighting.C:105-124)
// and from the numbering the C ABI fixes for particle records and fields
// (include/picgpu.h): cells in block order (x fastest) without the removed
// boxes; local faces -x, +x, -y, +y, -z, +z with their corners in
// right-hand outward order starting at the face's base point; tet
// 2 f + k = (cell centre, base point, corners k + 1 and k + 2 of face f);
// points merged across cyclic pairs; boundary faces in (cell, local face)
// order; one geometry class for a block of equal cells, the geometry of its
// first cell.
//
// The library has its own mesh code; the two agree because they state the
// same geometry, which the known-answer tests of tests/test_oracle_mesh.py
// check from first principles (volumes, barycentric round trips, the
// Laplacian of linear fields, partitions of unity).
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "picgpu.h"

namespace om {

// Corner q of cell (i, j, k) is grid point (i, j, k) + kBits[q].
static const int kBits[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
// Local faces -x, +x, -y, +y, -z, +z: corners in outward right-hand order.
static const int kFaceQ[6][4] = {{0, 4, 7, 3}, {1, 2, 6, 5}, {0, 1, 5, 4},
                                 {3, 7, 6, 2}, {0, 3, 2, 1}, {4, 5, 6, 7}};

// Tet-to-tet moves of the canonical hex.  A tet's vertex 0 is the cell
// centre, vertices 1..3 the corners tri[t][0..2].
struct TetTables {
    int tri[12][3];
    int inner_next[12][4];    // through the face opposite vertex i (1..3): the tet beyond
    int inner_src[12][4][4];  // its coordinate j comes from old coordinate src (-1: zero)
    int cross_next[12];       // through the cell face (opposite vertex 0): the tet in the neighbour
    int cross_src[12][4];
};

inline TetTables tet_tables() {
    TetTables T{};
    for (int f = 0; f < 6; ++f)
        for (int k = 0; k < 2; ++k) {
            const int t = 2 * f + k;
            T.tri[t][0] = kFaceQ[f][0];
            T.tri[t][1] = kFaceQ[f][1 + k];
            T.tri[t][2] = kFaceQ[f][2 + k];
        }
    auto vertex = [&](int t, int v) { return v == 0 ? -1 : T.tri[t][v - 1]; };  // -1: the centre
    auto has = [&](int t, int corner) {
        return T.tri[t][0] == corner || T.tri[t][1] == corner || T.tri[t][2] == corner;
    };
    for (int t = 0; t < 12; ++t) {
        T.inner_next[t][0] = -1;
        for (int j = 0; j < 4; ++j) T.inner_src[t][0][j] = -1;
        for (int i = 1; i <= 3; ++i) {
            // the shared face keeps the centre and the two corners other than vertex i
            int keep[2], nk = 0;
            for (int v = 1; v <= 3; ++v)
                if (v != i) keep[nk++] = vertex(t, v);
            int u = -1;
            for (int c = 0; c < 12 && u < 0; ++c)
                if (c != t && has(c, keep[0]) && has(c, keep[1])) u = c;
            if (u < 0) throw std::runtime_error("oracle mesh: tet without a neighbour");
            T.inner_next[t][i] = u;
            for (int j = 0; j < 4; ++j) {
                T.inner_src[t][i][j] = -1;
                for (int v = 0; v < 4; ++v)
                    if (v != i && vertex(t, v) == vertex(u, j)) T.inner_src[t][i][j] = v;
            }
        }
        // across the cell face: the neighbour sees the same triangle from its
        // opposite face; corners map by flipping the face-normal bit
        const int f = t / 2, axis = f / 2;
        int image[3];
        for (int v = 0; v < 3; ++v) {
            int b[3] = {kBits[T.tri[t][v]][0], kBits[T.tri[t][v]][1], kBits[T.tri[t][v]][2]};
            b[axis] = 1 - b[axis];
            for (int q = 0; q < 8; ++q)
                if (kBits[q][0] == b[0] && kBits[q][1] == b[1] && kBits[q][2] == b[2]) image[v] = q;
        }
        T.cross_next[t] = -1;
        for (int u = 2 * (f ^ 1); u < 2 * (f ^ 1) + 2; ++u)
            if (has(u, image[0]) && has(u, image[1]) && has(u, image[2])) T.cross_next[t] = u;
        if (T.cross_next[t] < 0) throw std::runtime_error("oracle mesh: cell-face triangles do not match");
        const int u = T.cross_next[t];
        T.cross_src[t][0] = -1;
        for (int j = 0; j < 3; ++j)
            for (int v = 0; v < 3; ++v)
                if (T.tri[u][j] == image[v]) T.cross_src[t][j + 1] = v + 1;
    }
    return T;
}

struct Patch {
    picgpu_patch p;
    double area = 0.0;
    int n_faces = 0;
};

struct BFace {
    int cell, local_face, patch;
    double normal[3];    // outward unit normal
    double area;
    double centre[3];
    double delta;        // cell centre to face centre
};

struct Mesh {
    int n[3] = {0, 0, 0};
    int cyclic[3] = {0, 0, 0};
    int empty[3] = {0, 0, 0};
    double mesh_centre[3] = {0, 0, 0};
    int n_cells = 0, n_points = 0, n_grid_points = 0;
    std::vector<double> grid_pts;   // 3 per grid point (i fastest)
    std::vector<int> cell_ijk;      // 3 per cell
    std::vector<int> grid_cell;     // block cell -> cell or -1
    std::vector<int> cell_gpt;      // 8 per cell: grid points of the corners
    std::vector<int> cell_pt;       // 8 per cell: merged points of the corners
    std::vector<double> cc, vol;
    std::vector<int> nbr;           // 6 per cell: neighbour, or -(patch + 1)
    std::vector<Patch> patches;     // the 6 block sides, then the boxes
    int n_classes = 1;
    std::vector<int> cell_class;
    std::vector<double> cls_offset;   // per class: 8 corners - centre
    std::vector<double> cls_tetinv;   // per class and tet: 3 rows, y_{1..3} = row . (x - centre)
    std::vector<double> cls_fnormal;  // per class: 6 outward unit normals
    std::vector<double> cls_farea;    // per class: 6 face areas
    std::vector<double> lap_off, lap_diag, ip_weight;
    std::vector<BFace> bfaces;
    std::vector<int> cell_bface;
    int has_dirichlet = 0;
    std::vector<double> vw_weight;    // 8 per cell (VolumeWeighting.C:44-89)
    std::vector<int> pi_start, pi_src;
    std::vector<double> pi_w;
    TetTables tt;
};

inline void vcross(const double* a, const double* b, double* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
inline double vdot(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline double vmag(const double* a) { return std::sqrt(vdot(a, a)); }

inline std::string check(const picgpu_mesh_desc& d) {
    for (int a = 0; a < 3; ++a) {
        if (d.n[a] < 1 || !(d.length[a] > 0)) return "mesh: bad size";
        const int k0 = d.side[2 * a].kind, k1 = d.side[2 * a + 1].kind;
        for (int k : {k0, k1})
            if (k < PICGPU_PATCH_CYCLIC || k > PICGPU_PATCH_CIRCUIT) return "mesh: unknown patch kind";
        if ((k0 == PICGPU_PATCH_CYCLIC) != (k1 == PICGPU_PATCH_CYCLIC)) return "mesh: unpaired cyclic side";
        if ((k0 == PICGPU_PATCH_EMPTY) != (k1 == PICGPU_PATCH_EMPTY)) return "mesh: unpaired empty side";
        if (k0 == PICGPU_PATCH_EMPTY && d.n[a] != 1) return "mesh: empty direction thicker than one cell";
    }
    if (d.n_boxes < 0 || d.n_boxes > PICGPU_MAX_BOXES) return "mesh: bad box count";
    for (int b = 0; b < d.n_boxes; ++b) {
        for (int a = 0; a < 3; ++a)
            if (d.box[b].lo[a] < 0 || d.box[b].hi[a] > d.n[a] || d.box[b].lo[a] >= d.box[b].hi[a])
                return "mesh: box out of range";
        const int k = d.box[b].patch.kind;
        if (k == PICGPU_PATCH_CYCLIC || k == PICGPU_PATCH_EMPTY) return "mesh: cyclic or empty box";
    }
    if (double(d.n[0]) * d.n[1] * d.n[2] > 1.5e8) return "mesh: too many cells";
    return "";
}

inline Mesh build(const picgpu_mesh_desc& d) {
    const std::string err = check(d);
    if (!err.empty()) throw std::runtime_error(err);
    Mesh m;
    m.tt = tet_tables();
    const int nx = d.n[0], ny = d.n[1], nz = d.n[2];
    for (int a = 0; a < 3; ++a) {
        m.n[a] = d.n[a];
        m.cyclic[a] = d.side[2 * a].kind == PICGPU_PATCH_CYCLIC;
        m.empty[a] = d.side[2 * a].kind == PICGPU_PATCH_EMPTY;
        m.mesh_centre[a] = d.origin[a] + 0.5 * d.length[a];
    }
    // grid points x_i = origin + length * i / n
    m.n_grid_points = (nx + 1) * (ny + 1) * (nz + 1);
    m.grid_pts.resize(3 * size_t(m.n_grid_points));
    auto gid = [&](int i, int j, int k) { return i + (nx + 1) * (j + (ny + 1) * k); };
    for (int k = 0; k <= nz; ++k)
        for (int j = 0; j <= ny; ++j)
            for (int i = 0; i <= nx; ++i) {
                const int ijk[3] = {i, j, k};
                for (int a = 0; a < 3; ++a)
                    m.grid_pts[3 * size_t(gid(i, j, k)) + a] = d.origin[a] + d.length[a] * double(ijk[a]) / double(d.n[a]);
            }
    // merged points: a cyclic direction identifies index n with 0
    const int mi = m.cyclic[0] ? nx : nx + 1, mj = m.cyclic[1] ? ny : ny + 1, mk = m.cyclic[2] ? nz : nz + 1;
    m.n_points = mi * mj * mk;
    auto mid = [&](int i, int j, int k) { return (i % mi) + mi * ((j % mj) + mj * (k % mk)); };
    // cells: the block minus the boxes, x fastest
    const long nb = long(nx) * ny * nz;
    std::vector<int> box_of(nb, -1);
    for (int b = 0; b < d.n_boxes; ++b)
        for (int k = d.box[b].lo[2]; k < d.box[b].hi[2]; ++k)
            for (int j = d.box[b].lo[1]; j < d.box[b].hi[1]; ++j)
                for (int i = d.box[b].lo[0]; i < d.box[b].hi[0]; ++i) box_of[i + long(nx) * (j + long(ny) * k)] = b;
    m.grid_cell.assign(nb, -1);
    for (long g = 0; g < nb; ++g)
        if (box_of[g] < 0) m.grid_cell[g] = m.n_cells++;
    if (m.n_cells == 0) throw std::runtime_error("mesh: every cell removed");
    const int nc = m.n_cells;
    m.patches.resize(6 + d.n_boxes);
    for (int s = 0; s < 6; ++s) m.patches[s].p = d.side[s];
    for (int b = 0; b < d.n_boxes; ++b) m.patches[6 + b].p = d.box[b].patch;
    m.cell_ijk.resize(3 * size_t(nc));
    m.cell_gpt.resize(8 * size_t(nc));
    m.cell_pt.resize(8 * size_t(nc));
    m.cc.resize(3 * size_t(nc));
    m.nbr.resize(6 * size_t(nc));
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const int c = m.grid_cell[i + long(nx) * (j + long(ny) * k)];
                if (c < 0) continue;
                const int ijk[3] = {i, j, k};
                double sum[3] = {0.0, 0.0, 0.0};
                for (int q = 0; q < 8; ++q) {
                    const int g = gid(i + kBits[q][0], j + kBits[q][1], k + kBits[q][2]);
                    m.cell_gpt[8 * size_t(c) + q] = g;
                    m.cell_pt[8 * size_t(c) + q] = mid(i + kBits[q][0], j + kBits[q][1], k + kBits[q][2]);
                    for (int a = 0; a < 3; ++a) sum[a] += m.grid_pts[3 * size_t(g) + a];
                }
                for (int a = 0; a < 3; ++a) {
                    m.cell_ijk[3 * size_t(c) + a] = ijk[a];
                    m.cc[3 * size_t(c) + a] = sum[a] / 8.0;   // centroid of a parallelepiped
                }
                for (int f = 0; f < 6; ++f) {
                    const int a = f / 2;
                    int q[3] = {i, j, k};
                    q[a] += (f & 1) ? 1 : -1;
                    int code;
                    if (q[a] < 0 || q[a] >= d.n[a]) {
                        if (!m.cyclic[a]) {
                            code = -(f + 1);                 // the block side of this face
                            m.nbr[6 * size_t(c) + f] = code;
                            continue;
                        }
                        q[a] = (q[a] + d.n[a]) % d.n[a];
                    }
                    const long g = q[0] + long(nx) * (q[1] + long(ny) * q[2]);
                    code = box_of[g] >= 0 ? -(6 + box_of[g] + 1) : m.grid_cell[g];
                    m.nbr[6 * size_t(c) + f] = code;
                }
            }
    // one geometry class: the corner offsets of the first cell
    m.cell_class.assign(nc, 0);
    m.cls_offset.resize(24);
    for (int q = 0; q < 8; ++q)
        for (int a = 0; a < 3; ++a)
            m.cls_offset[3 * q + a] = m.grid_pts[3 * size_t(m.cell_gpt[q]) + a] - m.cc[a];
    const double* off = m.cls_offset.data();
    // barycentric rows of each tet: with corners A, B, C relative to the
    // centre, x = y1 A + y2 B + y3 C solves to y1 = (B x C).x / det, ...
    m.cls_tetinv.resize(108);
    double cell_volume = 0.0;
    for (int t = 0; t < 12; ++t) {
        const double* A = off + 3 * m.tt.tri[t][0];
        const double* B = off + 3 * m.tt.tri[t][1];
        const double* C = off + 3 * m.tt.tri[t][2];
        double r1[3], r2[3], r3[3];
        vcross(B, C, r1);
        vcross(C, A, r2);
        vcross(A, B, r3);
        const double det = vdot(A, r1);
        if (!(std::fabs(det) > 0.0)) throw std::runtime_error("mesh: degenerate tet");
        for (int a = 0; a < 3; ++a) {
            m.cls_tetinv[9 * t + a] = r1[a] / det;
            m.cls_tetinv[9 * t + 3 + a] = r2[a] / det;
            m.cls_tetinv[9 * t + 6 + a] = r3[a] / det;
        }
        cell_volume += std::fabs(det) / 6.0;
    }
    m.vol.assign(nc, cell_volume);
    // faces: area vector of a planar quad = (diagonal 02 x diagonal 13) / 2
    m.cls_fnormal.resize(18);
    m.cls_farea.resize(6);
    double fcentre[6][3];
    for (int f = 0; f < 6; ++f) {
        const double* p[4];
        for (int v = 0; v < 4; ++v) p[v] = off + 3 * kFaceQ[f][v];
        const double d02[3] = {p[2][0] - p[0][0], p[2][1] - p[0][1], p[2][2] - p[0][2]};
        const double d13[3] = {p[3][0] - p[1][0], p[3][1] - p[1][1], p[3][2] - p[1][2]};
        double S[3];
        vcross(d02, d13, S);
        const double area = 0.5 * vmag(S);
        m.cls_farea[f] = area;
        for (int a = 0; a < 3; ++a) {
            m.cls_fnormal[3 * f + a] = S[a] / (2.0 * area);
            fcentre[f][a] = 0.25 * (p[0][a] + p[1][a] + p[2][a] + p[3][a]);
        }
    }
    // Gauss Laplacian on the orthogonal mesh: |S| / |d| per coupled face,
    // |S| / |d_b| on fixedValue boundary faces; linear face interpolation
    // weight of the owner w_P = |d_N| / (|d_P| + |d_N|)
    m.lap_off.assign(6 * size_t(nc), 0.0);
    m.lap_diag.assign(nc, 0.0);
    m.ip_weight.assign(6 * size_t(nc), 0.5);
    m.cell_bface.assign(6 * size_t(nc), -1);
    for (int c = 0; c < nc; ++c)
        for (int f = 0; f < 6; ++f) {
            const int code = m.nbr[6 * size_t(c) + f];
            const double area = m.cls_farea[f];
            const double dP = vmag(fcentre[f]);
            if (code >= 0) {
                const double dN = vmag(fcentre[f ^ 1]);
                const double coef = area / (dP + dN);
                m.lap_off[6 * size_t(c) + f] = coef;
                m.lap_diag[c] -= coef;
                m.ip_weight[6 * size_t(c) + f] = dN / (dP + dN);
                continue;
            }
            Patch& P = m.patches[-code - 1];
            P.area += area;
            P.n_faces += 1;
            if (P.p.kind == PICGPU_PATCH_EMPTY) continue;
            BFace b{};
            b.cell = c;
            b.local_face = f;
            b.patch = -code - 1;
            b.area = area;
            b.delta = dP;
            for (int a = 0; a < 3; ++a) {
                b.normal[a] = m.cls_fnormal[3 * f + a];
                b.centre[a] = m.cc[3 * size_t(c) + a] + fcentre[f][a];
            }
            m.cell_bface[6 * size_t(c) + f] = int(m.bfaces.size());
            const int k = P.p.kind;
            if ((k == PICGPU_PATCH_ABSORB || k == PICGPU_PATCH_WALL || k == PICGPU_PATCH_CIRCUIT) &&
                P.p.phi_bc == PICGPU_PHI_FIXED_VALUE) {
                m.lap_diag[c] -= area / dP;
                m.has_dirichlet = 1;
            }
            m.bfaces.push_back(b);
        }
    // VolumeWeighting: a point's charge goes to the cells around it in
    // proportion to the corner-centre distance (not its inverse)
    m.vw_weight.assign(8 * size_t(nc), 0.0);
    std::vector<double> around(m.n_points, 0.0);
    for (int c = 0; c < nc; ++c)
        for (int q = 0; q < 8; ++q) {
            const double w = vmag(off + 3 * q);
            m.vw_weight[8 * size_t(c) + q] = w;
            around[m.cell_pt[8 * size_t(c) + q]] += w;
        }
    for (int c = 0; c < nc; ++c)
        for (int q = 0; q < 8; ++q) m.vw_weight[8 * size_t(c) + q] /= around[m.cell_pt[8 * size_t(c) + q]];
    // cell -> point interpolation (interpolationCellPoint's weights): inverse
    // distance to the boundary face centres at points on non-coupled,
    // non-empty patches, else to the surrounding cell centres
    std::vector<std::vector<std::pair<int, double>>> from(m.n_points);
    std::vector<char> boundary_point(m.n_points, 0);
    for (const BFace& b : m.bfaces)
        for (int v = 0; v < 4; ++v) boundary_point[m.cell_pt[8 * size_t(b.cell) + kFaceQ[b.local_face][v]]] = 1;
    for (size_t bi = 0; bi < m.bfaces.size(); ++bi) {
        const BFace& b = m.bfaces[bi];
        for (int v = 0; v < 4; ++v) {
            const int q = kFaceQ[b.local_face][v];
            const int g = m.cell_gpt[8 * size_t(b.cell) + q];
            const double r[3] = {m.grid_pts[3 * size_t(g)] - b.centre[0], m.grid_pts[3 * size_t(g) + 1] - b.centre[1],
                                 m.grid_pts[3 * size_t(g) + 2] - b.centre[2]};
            from[m.cell_pt[8 * size_t(b.cell) + q]].push_back({-(int(bi) + 1), 1.0 / vmag(r)});
        }
    }
    for (int c = 0; c < nc; ++c)
        for (int q = 0; q < 8; ++q) {
            const int p = m.cell_pt[8 * size_t(c) + q];
            if (!boundary_point[p]) from[p].push_back({c, 1.0 / vmag(off + 3 * q)});
        }
    m.pi_start.assign(m.n_points + 1, 0);
    for (int p = 0; p < m.n_points; ++p) {
        m.pi_start[p + 1] = m.pi_start[p] + int(from[p].size());
        double s = 0.0;
        for (const auto& e : from[p]) s += e.second;
        for (const auto& e : from[p]) {
            m.pi_src.push_back(e.first);
            m.pi_w.push_back(e.second / s);
        }
    }
    return m;
}

inline int grid_point_id(const Mesh& m, int i, int j, int k) { return i + (m.n[0] + 1) * (j + (m.n[1] + 1) * k); }

// Barycentric coordinates 1..3 of the point x in tet t of cell c.
inline void tet_coords(const Mesh& m, int c, int t, const double* x, double* y) {
    const double* row = &m.cls_tetinv[(size_t(m.cell_class[c]) * 12 + t) * 9];
    const double r[3] = {x[0] - m.cc[3 * size_t(c)], x[1] - m.cc[3 * size_t(c) + 1], x[2] - m.cc[3 * size_t(c) + 2]};
    for (int k = 0; k < 3; ++k) y[k] = row[3 * k] * r[0] + row[3 * k + 1] * r[1] + row[3 * k + 2] * r[2];
}

// mesh.findCell for the block: the cell (by its block indices) holding x, and
// in it the tet whose smallest barycentric coordinate is largest, with the
// coordinates clamped to >= 0 and renormalised.  Returns cell 12 + tet, or -1
// when x lies outside the block (beyond 1e-9 of a cell) or in a removed box.
inline long long locate(const Mesh& m, const double* x, double* y) {
    const int top = grid_point_id(m, m.n[0], m.n[1], m.n[2]);
    long long g = 0, stride = 1;
    for (int a = 0; a < 3; ++a) {
        const double lo = m.grid_pts[a], hi = m.grid_pts[3 * size_t(top) + a];
        const double u = (x[a] - lo) / (hi - lo) * m.n[a];
        if (!(u >= -1e-9 && u <= m.n[a] + 1e-9)) return -1;
        const int i = std::min(std::max(int(std::floor(u)), 0), m.n[a] - 1);
        g += stride * i;
        stride *= m.n[a];
    }
    const int c = m.grid_cell[g];
    if (c < 0) return -1;
    int best = 0;
    double best_min = -1e300, q[3] = {0.0, 0.0, 0.0};
    for (int t = 0; t < 12; ++t) {
        double w[3];
        tet_coords(m, c, t, x, w);
        const double lowest = std::fmin(std::fmin(1.0 - w[0] - w[1] - w[2], w[0]), std::fmin(w[1], w[2]));
        if (lowest > best_min) {
            best_min = lowest;
            best = t;
            q[0] = w[0];
            q[1] = w[1];
            q[2] = w[2];
        }
    }
    if (best_min < -1e-9) return -1;
    const double all[4] = {std::fmax(1.0 - q[0] - q[1] - q[2], 0.0), std::fmax(q[0], 0.0), std::fmax(q[1], 0.0),
                           std::fmax(q[2], 0.0)};
    const double sum = all[0] + all[1] + all[2] + all[3];
    for (int k = 0; k < 3; ++k) y[k] = all[k + 1] / sum;
    return 12LL * c + best;
}

// x in cell c (known): the tet whose smallest barycentric coordinate is
// largest, coordinates clamped to >= 0 and renormalised, as locate() does
// once it has the cell.  Returns cell 12 + tet.
inline long long locate_in_cell(const Mesh& m, int c, const double* x, double* y) {
    int best = 0;
    double best_min = -1e300, q[3] = {0.0, 0.0, 0.0};
    for (int t = 0; t < 12; ++t) {
        double w[3];
        tet_coords(m, c, t, x, w);
        const double lowest = std::fmin(std::fmin(1.0 - w[0] - w[1] - w[2], w[0]), std::fmin(w[1], w[2]));
        if (lowest > best_min) {
            best_min = lowest;
            best = t;
            q[0] = w[0];
            q[1] = w[1];
            q[2] = w[2];
        }
    }
    const double all[4] = {std::fmax(1.0 - q[0] - q[1] - q[2], 0.0), std::fmax(q[0], 0.0), std::fmax(q[1], 0.0),
                           std::fmax(q[2], 0.0)};
    const double sum = all[0] + all[1] + all[2] + all[3];
    for (int k = 0; k < 3; ++k) y[k] = all[k + 1] / sum;
    return 12LL * c + best;
}

// The point of barycentric coordinates y (1..3) in tet `tet` (cell 12 + t).
inline void position(const Mesh& m, long long tet, const double* y, double* x) {
    const long long c = tet / 12;
    const int t = int(tet % 12);
    const double* off = &m.cls_offset[size_t(m.cell_class[c]) * 24];
    for (int a = 0; a < 3; ++a)
        x[a] = m.cc[3 * size_t(c) + a] + y[0] * off[3 * m.tt.tri[t][0] + a] + y[1] * off[3 * m.tt.tri[t][1] + a] +
               y[2] * off[3 * m.tt.tri[t][2] + a];
}

// Volume of tet t of class `cls`.
inline double tet_volume(const Mesh& m, int cls, int t) {
    const double* off = &m.cls_offset[size_t(cls) * 24];
    double bc[3];
    vcross(off + 3 * m.tt.tri[t][1], off + 3 * m.tt.tri[t][2], bc);
    return std::fabs(vdot(off + 3 * m.tt.tri[t][0], bc)) / 6.0;
}

// The emitting triangles of a patch (ParticleEmitter::initilizeParticleEmitter,
// ParticleEmitter.C:54-139): each boundary face of the patch split into the
// face triangles of its two tets, with the cumulative triangle areas.
struct PatchTriangles {
    std::vector<int> cell, tet;
    std::vector<double> normal, centre;
    std::vector<double> cum;
    double area = 0.0;
};

inline PatchTriangles patch_triangles(const Mesh& m, int patch) {
    PatchTriangles T;
    T.cum.push_back(0.0);
    for (const BFace& b : m.bfaces) {
        if (b.patch != patch) continue;
        T.area += b.area;
        const double* off = &m.cls_offset[size_t(m.cell_class[b.cell]) * 24];
        for (int k = 0; k < 2; ++k) {
            const int t = 2 * b.local_face + k;
            const double* A = off + 3 * m.tt.tri[t][0];
            const double* B = off + 3 * m.tt.tri[t][1];
            const double* C = off + 3 * m.tt.tri[t][2];
            const double u[3] = {B[0] - A[0], B[1] - A[1], B[2] - A[2]};
            const double v[3] = {C[0] - A[0], C[1] - A[1], C[2] - A[2]};
            double w[3];
            vcross(u, v, w);
            T.cell.push_back(b.cell);
            T.tet.push_back(t);
            for (int a = 0; a < 3; ++a) {
                T.normal.push_back(b.normal[a]);
                T.centre.push_back(b.centre[a]);
            }
            T.cum.push_back(T.cum.back() + 0.5 * vmag(w));
        }
    }
    return T;
}

}  // namespace om
