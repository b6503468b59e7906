// hexmesh.hpp -- hexahedral block mesh with OpenFOAM-style tet decomposition.
//
// This is the mesh layer the particle hot path runs on (the role polyMesh,
// polyMeshTetDecomposition and the cell/point addressing of OpenFOAM play for
// picFoam).  It is host C++ only and header-only so that the CUDA library and
// the CPU oracle build the identical mesh from one picgpu_mesh_desc.
//
// Tet decomposition (the scheme described by Macpherson, Nordin & Weller,
// Commun. Numer. Meth. Engng 25 (2009) 263, as used by OpenFOAM's barycentric
// tracking and by picFoam's VolumeWeighting charge model,
// PICMCCFVM/submodels/ChargeDistribution/VolumeWeighting/VolumeWeighting.C:105-124):
// every quad face is fanned from its first point into two triangles; a tet is
// (cell centre, triangle point 0, 1, 2).  Barycentric coordinate 0 belongs to
// the cell centre, 1..3 to the triangle points.  A hex has 6 faces x 2 = 12
// tets; tet t lies on local face t/2.
//
// Two cells sharing a face split it along the same diagonal (the local face
// tables below are chosen so), so crossing a cell face maps the three triangle
// coordinates across unchanged up to a fixed permutation.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <array>
#include <vector>

#include "picgpu.h"

namespace pg {

// ---------------------------------------------------------------- local hex --
// Corner c of a hex cell sits at offset (bx, by, bz) of the cell's (i, j, k).
static const int kCornerBits[8][3] = {
    {0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
    {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

// Local faces -x, +x, -y, +y, -z, +z; points ordered so the right-hand normal
// points out of the cell.
static const int kFaceCorners[6][4] = {
    {0, 4, 7, 3}, {1, 2, 6, 5}, {0, 1, 5, 4},
    {3, 7, 6, 2}, {0, 3, 2, 1}, {4, 5, 6, 7}};

struct TetTables {
    int tri[12][3];          // local corners of the face triangle of tet t
    // crossing tet face i (1..3, opposite barycentric vertex i) inside the cell
    int inner_next[12][4];   // neighbouring tet (entry 0 unused)
    int inner_src[12][4][4]; // new coord j <- old coord src (-1: zero)
    // crossing tet face 0 (the cell face) into the neighbour cell
    int cross_next[12];      // local tet in the neighbour
    int cross_src[12][4];    // new coord j <- old coord src (j = 1..3; [0] = -1)
};

inline TetTables make_tet_tables() {
    TetTables T{};
    for (int t = 0; t < 12; ++t) {
        const int f = t / 2, k = t % 2;
        T.tri[t][0] = kFaceCorners[f][0];
        T.tri[t][1] = kFaceCorners[f][k + 1];
        T.tri[t][2] = kFaceCorners[f][k + 2];
    }
    // vertex list of tet t: index 0 = cell centre (-1), 1..3 = corners
    auto vert = [&](int t, int i) { return i == 0 ? -1 : T.tri[t][i - 1]; };
    for (int t = 0; t < 12; ++t) {
        T.inner_next[t][0] = -1;
        for (int a = 0; a < 4; ++a) T.inner_src[t][0][a] = -1;
        for (int i = 1; i <= 3; ++i) {
            // the face opposite vertex i holds the centre and the other two corners
            int e0 = -1, e1 = -1;
            for (int j = 1; j <= 3; ++j)
                if (j != i) { if (e0 < 0) e0 = vert(t, j); else e1 = vert(t, j); }
            int found = -1;
            for (int u = 0; u < 12; ++u) {
                if (u == t) continue;
                bool h0 = false, h1 = false;
                for (int j = 0; j < 3; ++j) {
                    h0 |= T.tri[u][j] == e0;
                    h1 |= T.tri[u][j] == e1;
                }
                if (h0 && h1) { found = u; break; }
            }
            if (found < 0) throw std::runtime_error("tet table: no neighbour tet");
            T.inner_next[t][i] = found;
            for (int j = 0; j < 4; ++j) {
                const int v = vert(found, j);
                int src = -1;
                for (int a = 0; a < 4; ++a)
                    if (a != i && vert(t, a) == v) src = a;
                T.inner_src[t][i][j] = src;  // -1 for the new vertex
            }
        }
    }
    // cell-face crossing: corner mapped by flipping the face-normal bit
    for (int t = 0; t < 12; ++t) {
        const int f = t / 2, d = f / 2;
        const int fn = f ^ 1;  // opposite local face of the neighbour
        int mapped[3];
        for (int j = 0; j < 3; ++j) {
            int b[3] = {kCornerBits[T.tri[t][j]][0], kCornerBits[T.tri[t][j]][1],
                        kCornerBits[T.tri[t][j]][2]};
            b[d] ^= 1;
            int c = -1;
            for (int q = 0; q < 8; ++q)
                if (kCornerBits[q][0] == b[0] && kCornerBits[q][1] == b[1] &&
                    kCornerBits[q][2] == b[2]) c = q;
            mapped[j] = c;
        }
        int found = -1;
        for (int u = 2 * fn; u < 2 * fn + 2; ++u) {
            int hits = 0;
            for (int j = 0; j < 3; ++j)
                for (int q = 0; q < 3; ++q) hits += T.tri[u][j] == mapped[q];
            if (hits == 3) found = u;
        }
        if (found < 0) throw std::runtime_error("tet table: face triangles disagree");
        T.cross_next[t] = found;
        T.cross_src[t][0] = -1;
        for (int j = 0; j < 3; ++j)
            for (int q = 0; q < 3; ++q)
                if (T.tri[found][j] == mapped[q]) T.cross_src[t][j + 1] = q + 1;
    }
    return T;
}

// ------------------------------------------------------------------ mesh ----
struct Patch {
    picgpu_patch p;
    double area = 0.0;   // total face area
    int n_faces = 0;
};

// Boundary face on a non-coupled, non-empty patch.
struct BFace {
    int cell, local_face, patch;
    double normal[3];    // unit, out of the domain
    double area;
    double centre[3];
    double delta;        // cell centre -> face centre distance
};

struct HexMesh {
    int n[3] = {0, 0, 0};
    int cyclic[3] = {0, 0, 0};
    int empty[3] = {0, 0, 0};      // reduced-D direction (geometricD == -1)
    double mesh_centre[3] = {0, 0, 0};
    int n_cells = 0;
    int n_grid_points = 0;         // geometric points
    int n_points = 0;              // cyclic-merged points
    std::vector<double> grid_pts;  // 3 * n_grid_points
    std::vector<int> cell_ijk;     // 3 * n_cells
    std::vector<int> grid_cell;    // block cell -> cell id or -1
    std::vector<int> cell_gpt;     // 8 * n_cells geometric point ids
    std::vector<int> cell_pt;      // 8 * n_cells cyclic-merged point ids
    std::vector<double> cc;        // 3 * n_cells
    std::vector<double> vol;       // n_cells
    std::vector<int> nbr;          // 6 * n_cells: >= 0 cell, < 0: -(patch + 1)
    std::vector<Patch> patches;

    // geometry classes (cells congruent up to translation share one)
    int n_classes = 0;
    std::vector<int> cell_class;       // n_cells
    std::vector<double> cls_offset;    // class * 8 * 3: corner - centre
    std::vector<double> cls_tetinv;    // class * 12 * 9: rows of inverse of [a b c]
    std::vector<double> cls_fnormal;   // class * 6 * 3 unit outward
    std::vector<double> cls_farea;     // class * 6
    std::vector<double> cls_fcentre;   // class * 6 * 3 (relative to centre)

    // finite volume data (orthogonal hex mesh)
    std::vector<double> lap_off;    // 6 * n_cells: |S_f|/|d| for coupled faces, else 0
    std::vector<double> lap_diag;   // n_cells (negative)
    std::vector<double> ip_weight;  // 6 * n_cells: owner weight of linear face interpolation
    std::vector<BFace> bfaces;
    std::vector<int> cell_bface;    // 6 * n_cells: boundary face id or -1
    int has_dirichlet = 0;

    // cell -> point charge weights (VolumeWeighting.C:44-89): distance weights
    std::vector<double> vw_weight;  // 8 * n_cells

    // point interpolation of cell/boundary values (CSR over merged points)
    std::vector<int> pi_start;      // n_points + 1
    std::vector<int> pi_src;        // >= 0 cell, < 0: -(bface + 1)
    std::vector<double> pi_w;

    // merged point -> the cell-corner slots (9 c + 1 + corner) that touch it
    std::vector<int> pc_start;      // n_points + 1
    std::vector<int> pc_slot;

    TetTables tt;
};

inline int grid_point_id(const HexMesh& m, int i, int j, int k) {
    return i + (m.n[0] + 1) * (j + (m.n[1] + 1) * k);
}

inline int merged_point_id(const HexMesh& m, int i, int j, int k) {
    const int ni = m.cyclic[0] ? m.n[0] : m.n[0] + 1;
    const int nj = m.cyclic[1] ? m.n[1] : m.n[1] + 1;
    if (m.cyclic[0]) i %= m.n[0];
    if (m.cyclic[1]) j %= m.n[1];
    if (m.cyclic[2]) k %= m.n[2];
    return i + ni * (j + nj * k);
}

inline void cross3(const double* a, const double* b, double* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
inline double dot3(const double* a, const double* b) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
inline double norm3(const double* a) { return std::sqrt(dot3(a, a)); }

inline std::string validate_desc(const picgpu_mesh_desc& d) {
    for (int a = 0; a < 3; ++a) {
        if (d.n[a] < 1) return "mesh: cell count must be >= 1 in every direction";
        if (!(d.length[a] > 0)) return "mesh: length must be > 0";
        const int k0 = d.side[2 * a].kind, k1 = d.side[2 * a + 1].kind;
        if ((k0 == PICGPU_PATCH_CYCLIC) != (k1 == PICGPU_PATCH_CYCLIC))
            return "mesh: cyclic sides must come in pairs";
        if ((k0 == PICGPU_PATCH_EMPTY) != (k1 == PICGPU_PATCH_EMPTY))
            return "mesh: empty sides must come in pairs";
        if (k0 == PICGPU_PATCH_EMPTY && d.n[a] != 1)
            return "mesh: an empty direction must be one cell thick";
        for (int s = 0; s < 2; ++s) {
            const int k = d.side[2 * a + s].kind;
            if (k < PICGPU_PATCH_CYCLIC || k > PICGPU_PATCH_CIRCUIT)
                return "mesh: unknown patch kind";
        }
    }
    if (d.n_boxes < 0 || d.n_boxes > PICGPU_MAX_BOXES) return "mesh: bad box count";
    for (int b = 0; b < d.n_boxes; ++b) {
        const picgpu_box& bx = d.box[b];
        for (int a = 0; a < 3; ++a)
            if (bx.lo[a] < 0 || bx.hi[a] > d.n[a] || bx.lo[a] >= bx.hi[a])
                return "mesh: box out of range";
        if (bx.patch.kind == PICGPU_PATCH_CYCLIC || bx.patch.kind == PICGPU_PATCH_EMPTY)
            return "mesh: a box patch cannot be cyclic or empty";
    }
    const double ncell = double(d.n[0]) * d.n[1] * d.n[2];
    if (ncell > 1.5e8) return "mesh: more than 1.5e8 cells";
    return "";
}

// Build the mesh.  Throws std::runtime_error on invalid input.
inline HexMesh build_hex_mesh(const picgpu_mesh_desc& d) {
    const std::string err = validate_desc(d);
    if (!err.empty()) throw std::runtime_error(err);
    HexMesh m;
    m.tt = make_tet_tables();
    for (int a = 0; a < 3; ++a) {
        m.n[a] = d.n[a];
        m.cyclic[a] = d.side[2 * a].kind == PICGPU_PATCH_CYCLIC;
        m.empty[a] = d.side[2 * a].kind == PICGPU_PATCH_EMPTY;
        m.mesh_centre[a] = d.origin[a] + 0.5 * d.length[a];
    }
    const int nx = d.n[0], ny = d.n[1], nz = d.n[2];
    // points
    m.n_grid_points = (nx + 1) * (ny + 1) * (nz + 1);
    m.grid_pts.resize(3 * size_t(m.n_grid_points));
    for (int k = 0; k <= nz; ++k)
        for (int j = 0; j <= ny; ++j)
            for (int i = 0; i <= nx; ++i) {
                const int p = grid_point_id(m, i, j, k);
                const int ijk[3] = {i, j, k};
                for (int a = 0; a < 3; ++a)
                    m.grid_pts[3 * size_t(p) + a] =
                        d.origin[a] + d.length[a] * double(ijk[a]) / double(d.n[a]);
            }
    m.n_points = (m.cyclic[0] ? nx : nx + 1) * (m.cyclic[1] ? ny : ny + 1) *
                 (m.cyclic[2] ? nz : nz + 1);
    // cells
    const size_t nblock = size_t(nx) * ny * nz;
    m.grid_cell.assign(nblock, 0);
    for (int b = 0; b < d.n_boxes; ++b) {
        const picgpu_box& bx = d.box[b];
        for (int k = bx.lo[2]; k < bx.hi[2]; ++k)
            for (int j = bx.lo[1]; j < bx.hi[1]; ++j)
                for (int i = bx.lo[0]; i < bx.hi[0]; ++i)
                    m.grid_cell[i + size_t(nx) * (j + size_t(ny) * k)] = -(b + 1);
    }
    int nc = 0;
    std::vector<int> cell_box(nblock, -1);
    for (size_t g = 0; g < nblock; ++g) {
        if (m.grid_cell[g] < 0) { cell_box[g] = -m.grid_cell[g] - 1; m.grid_cell[g] = -1; }
        else m.grid_cell[g] = nc++;
    }
    if (nc == 0) throw std::runtime_error("mesh: every cell removed");
    m.n_cells = nc;
    m.cell_ijk.resize(3 * size_t(nc));
    m.cell_gpt.resize(8 * size_t(nc));
    m.cell_pt.resize(8 * size_t(nc));
    m.cc.resize(3 * size_t(nc));
    m.vol.resize(nc);
    m.nbr.resize(6 * size_t(nc));
    // patches: 6 sides then boxes
    m.patches.resize(6 + d.n_boxes);
    for (int s = 0; s < 6; ++s) m.patches[s].p = d.side[s];
    for (int b = 0; b < d.n_boxes; ++b) m.patches[6 + b].p = d.box[b].patch;

    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const size_t g = i + size_t(nx) * (j + size_t(ny) * k);
                const int c = m.grid_cell[g];
                if (c < 0) continue;
                m.cell_ijk[3 * size_t(c)] = i;
                m.cell_ijk[3 * size_t(c) + 1] = j;
                m.cell_ijk[3 * size_t(c) + 2] = k;
                double cen[3] = {0, 0, 0};
                for (int q = 0; q < 8; ++q) {
                    const int ii = i + kCornerBits[q][0], jj = j + kCornerBits[q][1],
                              kk = k + kCornerBits[q][2];
                    const int gp = grid_point_id(m, ii, jj, kk);
                    m.cell_gpt[8 * size_t(c) + q] = gp;
                    m.cell_pt[8 * size_t(c) + q] = merged_point_id(m, ii, jj, kk);
                    for (int a = 0; a < 3; ++a) cen[a] += m.grid_pts[3 * size_t(gp) + a];
                }
                for (int a = 0; a < 3; ++a) m.cc[3 * size_t(c) + a] = cen[a] / 8.0;
                const int ijk[3] = {i, j, k};
                for (int f = 0; f < 6; ++f) {
                    const int a = f / 2, s = f % 2;
                    int q[3] = {i, j, k};
                    q[a] += s ? 1 : -1;
                    int code;
                    if (q[a] < 0 || q[a] >= d.n[a]) {
                        if (m.cyclic[a]) {
                            q[a] = (q[a] + d.n[a]) % d.n[a];
                            code = m.grid_cell[q[0] + size_t(nx) * (q[1] + size_t(ny) * q[2])];
                        } else {
                            code = -(f + 1);  // block side patch f
                        }
                    } else {
                        const size_t gq = q[0] + size_t(nx) * (q[1] + size_t(ny) * q[2]);
                        code = m.grid_cell[gq];
                        if (code < 0) code = -(6 + cell_box[gq] + 1);
                    }
                    (void)ijk;
                    m.nbr[6 * size_t(c) + f] = code;
                }
            }

    // geometry classes
    m.cell_class.resize(nc);
    std::map<std::vector<long long>, int> classes;
    std::vector<int> class_rep;
    for (int c = 0; c < nc; ++c) {
        double off[24];
        double h = 0;
        for (int q = 0; q < 8; ++q)
            for (int a = 0; a < 3; ++a) {
                off[3 * q + a] = m.grid_pts[3 * size_t(m.cell_gpt[8 * size_t(c) + q]) + a] -
                                 m.cc[3 * size_t(c) + a];
                h = std::fmax(h, std::fabs(off[3 * q + a]));
            }
        std::vector<long long> key(24);
        for (int r = 0; r < 24; ++r) key[r] = std::llround(off[r] / h * 1e9);
        key.push_back(std::llround(std::log2(h) * 1e6));
        auto it = classes.find(key);
        if (it == classes.end()) {
            const int id = int(class_rep.size());
            classes.emplace(key, id);
            class_rep.push_back(c);
            m.cell_class[c] = id;
        } else {
            m.cell_class[c] = it->second;
        }
    }
    m.n_classes = int(class_rep.size());
    m.cls_offset.resize(size_t(m.n_classes) * 24);
    m.cls_tetinv.resize(size_t(m.n_classes) * 108);
    m.cls_fnormal.resize(size_t(m.n_classes) * 18);
    m.cls_farea.resize(size_t(m.n_classes) * 6);
    m.cls_fcentre.resize(size_t(m.n_classes) * 18);
    std::vector<double> cls_vol(m.n_classes);
    for (int cl = 0; cl < m.n_classes; ++cl) {
        const int c = class_rep[cl];
        double* off = &m.cls_offset[size_t(cl) * 24];
        for (int q = 0; q < 8; ++q)
            for (int a = 0; a < 3; ++a)
                off[3 * q + a] = m.grid_pts[3 * size_t(m.cell_gpt[8 * size_t(c) + q]) + a] -
                                 m.cc[3 * size_t(c) + a];
        double v = 0;
        for (int t = 0; t < 12; ++t) {
            const double* A = off + 3 * m.tt.tri[t][0];
            const double* B = off + 3 * m.tt.tri[t][1];
            const double* C = off + 3 * m.tt.tri[t][2];
            double bc[3], ca[3], ab[3];
            cross3(B, C, bc);
            cross3(C, A, ca);
            cross3(A, B, ab);
            const double det = dot3(A, bc);
            if (!(std::fabs(det) > 0)) throw std::runtime_error("mesh: degenerate tet");
            double* inv = &m.cls_tetinv[(size_t(cl) * 12 + t) * 9];
            for (int a = 0; a < 3; ++a) {
                inv[a] = bc[a] / det;
                inv[3 + a] = ca[a] / det;
                inv[6 + a] = ab[a] / det;
            }
            v += std::fabs(det) / 6.0;
        }
        cls_vol[cl] = v;
        for (int f = 0; f < 6; ++f) {
            const double* p0 = off + 3 * kFaceCorners[f][0];
            const double* p1 = off + 3 * kFaceCorners[f][1];
            const double* p2 = off + 3 * kFaceCorners[f][2];
            const double* p3 = off + 3 * kFaceCorners[f][3];
            double d02[3], d13[3], s[3];
            for (int a = 0; a < 3; ++a) { d02[a] = p2[a] - p0[a]; d13[a] = p3[a] - p1[a]; }
            cross3(d02, d13, s);
            const double area = 0.5 * norm3(s);
            m.cls_farea[size_t(cl) * 6 + f] = area;
            for (int a = 0; a < 3; ++a) {
                m.cls_fnormal[size_t(cl) * 18 + 3 * f + a] = s[a] / (2.0 * area);
                m.cls_fcentre[size_t(cl) * 18 + 3 * f + a] =
                    0.25 * (p0[a] + p1[a] + p2[a] + p3[a]);
            }
        }
    }
    for (int c = 0; c < nc; ++c) m.vol[c] = cls_vol[m.cell_class[c]];

    // finite-volume coefficients and boundary faces
    m.lap_off.assign(6 * size_t(nc), 0.0);
    m.lap_diag.assign(nc, 0.0);
    m.ip_weight.assign(6 * size_t(nc), 0.5);
    m.cell_bface.assign(6 * size_t(nc), -1);
    for (int c = 0; c < nc; ++c) {
        const int cl = m.cell_class[c];
        for (int f = 0; f < 6; ++f) {
            const int code = m.nbr[6 * size_t(c) + f];
            const double area = m.cls_farea[size_t(cl) * 6 + f];
            const double* fcr = &m.cls_fcentre[size_t(cl) * 18 + 3 * f];
            const double dP = norm3(fcr);
            if (code >= 0) {
                const int cln = m.cell_class[code];
                const double dN = norm3(&m.cls_fcentre[size_t(cln) * 18 + 3 * (f ^ 1)]);
                const double a = area / (dP + dN);
                m.lap_off[6 * size_t(c) + f] = a;
                m.lap_diag[c] -= a;
                m.ip_weight[6 * size_t(c) + f] = dN / (dP + dN);
            } else {
                const int patch = -code - 1;
                Patch& P = m.patches[patch];
                P.area += area;
                P.n_faces += 1;
                if (P.p.kind == PICGPU_PATCH_EMPTY) continue;
                BFace b{};
                b.cell = c;
                b.local_face = f;
                b.patch = patch;
                b.area = area;
                b.delta = dP;
                for (int a = 0; a < 3; ++a) {
                    b.normal[a] = m.cls_fnormal[size_t(cl) * 18 + 3 * f + a];
                    b.centre[a] = m.cc[3 * size_t(c) + a] + fcr[a];
                }
                m.cell_bface[6 * size_t(c) + f] = int(m.bfaces.size());
                const bool dirichlet = (P.p.kind == PICGPU_PATCH_ABSORB || P.p.kind == PICGPU_PATCH_WALL ||
                                        P.p.kind == PICGPU_PATCH_CIRCUIT) &&
                                       P.p.phi_bc == PICGPU_PHI_FIXED_VALUE;
                if (dirichlet) {
                    m.lap_diag[c] -= area / dP;
                    m.has_dirichlet = 1;
                }
                m.bfaces.push_back(b);
            }
        }
    }

    // VolumeWeighting charge weights: distance corner -> centre, normalised
    // over all cells sharing the (cyclic-merged) point.
    m.vw_weight.assign(8 * size_t(nc), 0.0);
    std::vector<double> wsum(m.n_points, 0.0);
    for (int c = 0; c < nc; ++c) {
        const double* off = &m.cls_offset[size_t(m.cell_class[c]) * 24];
        for (int q = 0; q < 8; ++q) {
            const double w = norm3(off + 3 * q);
            m.vw_weight[8 * size_t(c) + q] = w;
            wsum[m.cell_pt[8 * size_t(c) + q]] += w;
        }
    }
    for (int c = 0; c < nc; ++c)
        for (int q = 0; q < 8; ++q)
            m.vw_weight[8 * size_t(c) + q] /= wsum[m.cell_pt[8 * size_t(c) + q]];

    // point interpolation: inverse distance over boundary faces touching the
    // point when there are any (non-coupled, non-empty patches), else over the
    // cells around the point.
    std::vector<std::vector<std::pair<int, double>>> src(m.n_points);
    std::vector<char> on_boundary(m.n_points, 0);
    for (size_t b = 0; b < m.bfaces.size(); ++b) {
        const BFace& B = m.bfaces[b];
        for (int q = 0; q < 4; ++q) {
            const int corner = kFaceCorners[B.local_face][q];
            on_boundary[m.cell_pt[8 * size_t(B.cell) + corner]] = 1;
        }
    }
    for (size_t b = 0; b < m.bfaces.size(); ++b) {
        const BFace& B = m.bfaces[b];
        for (int q = 0; q < 4; ++q) {
            const int corner = kFaceCorners[B.local_face][q];
            const int gp = m.cell_gpt[8 * size_t(B.cell) + corner];
            double dv[3];
            for (int a = 0; a < 3; ++a) dv[a] = m.grid_pts[3 * size_t(gp) + a] - B.centre[a];
            src[m.cell_pt[8 * size_t(B.cell) + corner]].push_back({-(int(b) + 1), 1.0 / norm3(dv)});
        }
    }
    for (int c = 0; c < nc; ++c) {
        const double* off = &m.cls_offset[size_t(m.cell_class[c]) * 24];
        for (int q = 0; q < 8; ++q) {
            const int p = m.cell_pt[8 * size_t(c) + q];
            if (on_boundary[p]) continue;
            src[p].push_back({c, 1.0 / norm3(off + 3 * q)});
        }
    }
    m.pi_start.assign(m.n_points + 1, 0);
    for (int p = 0; p < m.n_points; ++p) m.pi_start[p + 1] = m.pi_start[p] + int(src[p].size());
    m.pi_src.resize(m.pi_start[m.n_points]);
    m.pi_w.resize(m.pi_start[m.n_points]);
    for (int p = 0; p < m.n_points; ++p) {
        double s = 0;
        for (auto& e : src[p]) s += e.second;
        int o = m.pi_start[p];
        for (auto& e : src[p]) { m.pi_src[o] = e.first; m.pi_w[o] = e.second / s; ++o; }
    }
    m.pc_start.assign(m.n_points + 1, 0);
    for (size_t k = 0; k < m.cell_pt.size(); ++k) m.pc_start[m.cell_pt[k] + 1]++;
    for (int p = 0; p < m.n_points; ++p) m.pc_start[p + 1] += m.pc_start[p];
    m.pc_slot.resize(m.cell_pt.size());
    {
        std::vector<int> fill(m.pc_start.begin(), m.pc_start.end() - 1);
        for (int c = 0; c < nc; ++c)
            for (int q = 0; q < 8; ++q) m.pc_slot[fill[m.cell_pt[8 * size_t(c) + q]]++] = 9 * c + 1 + q;
    }
    return m;
}

// Barycentric coordinates (1..3) of x in tet t of cell c.
inline void tet_coords(const HexMesh& m, int c, int t, const double* x, double* y) {
    const double* inv = &m.cls_tetinv[(size_t(m.cell_class[c]) * 12 + t) * 9];
    double r[3];
    for (int a = 0; a < 3; ++a) r[a] = x[a] - m.cc[3 * size_t(c) + a];
    for (int a = 0; a < 3; ++a) y[a] = inv[3 * a] * r[0] + inv[3 * a + 1] * r[1] + inv[3 * a + 2] * r[2];
}

// Locate x: returns tet id (cell*12 + t) or -1; bary gets coords 1..3.
inline long long locate(const HexMesh& m, const double* x, double* bary) {
    int ijk[3];
    for (int a = 0; a < 3; ++a) {
        const double lo = m.grid_pts[a];
        const double hi = m.grid_pts[3 * size_t(grid_point_id(m, m.n[0], m.n[1], m.n[2])) + a];
        double s = (x[a] - lo) / (hi - lo) * m.n[a];
        if (!(s >= -1e-9 && s <= m.n[a] + 1e-9)) return -1;
        int i = int(std::floor(s));
        if (i < 0) i = 0;
        if (i >= m.n[a]) i = m.n[a] - 1;
        ijk[a] = i;
    }
    const int c = m.grid_cell[ijk[0] + size_t(m.n[0]) * (ijk[1] + size_t(m.n[1]) * ijk[2])];
    if (c < 0) return -1;
    int best = -1;
    double best_min = -1e300, by[3] = {0, 0, 0};
    for (int t = 0; t < 12; ++t) {
        double y[3];
        tet_coords(m, c, t, x, y);
        const double y0 = 1.0 - y[0] - y[1] - y[2];
        const double mn = std::fmin(std::fmin(y0, y[0]), std::fmin(y[1], y[2]));
        if (mn > best_min) { best_min = mn; best = t; by[0] = y[0]; by[1] = y[1]; by[2] = y[2]; }
    }
    if (best_min < -1e-9) return -1;
    double y0 = 1.0 - by[0] - by[1] - by[2];
    double s = 0;
    double yy[4] = {std::fmax(y0, 0.0), std::fmax(by[0], 0.0), std::fmax(by[1], 0.0),
                    std::fmax(by[2], 0.0)};
    s = yy[0] + yy[1] + yy[2] + yy[3];
    for (int a = 0; a < 3; ++a) bary[a] = yy[a + 1] / s;
    return 12LL * c + best;
}

// The emitting triangles of one patch (ParticleEmitter::initilizeParticleEmitter,
// ParticleEmitter.C:54-139): each boundary face of the patch, in boundary-face
// order, split into the face triangles of its two tets; cum[0] = 0 and
// cum[i + 1] = cum[i] + area of triangle i; area = sum of the face areas.
struct PatchTriangles {
    std::vector<int> cell, tet;          // owner cell, local tet (2 face + k)
    std::vector<double> normal, centre;  // 3 per triangle: outward unit face normal, face centre
    std::vector<double> cum;
    double area = 0.0;
};

inline PatchTriangles patch_triangles(const HexMesh& m, int patch) {
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
            const double w[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
            const double a = 0.5 * std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
            T.cell.push_back(b.cell);
            T.tet.push_back(t);
            for (int q = 0; q < 3; ++q) {
                T.normal.push_back(b.normal[q]);
                T.centre.push_back(b.centre[q]);
            }
            T.cum.push_back(T.cum.back() + a);
        }
    }
    return T;
}

// Volume of tet t of geometry class cls (the cell centre and the three face
// points of its triangle): |a . (b x c)| / 6 with a, b, c the corner offsets.
inline double tet_volume(const HexMesh& m, int cls, int t) {
    const double* off = &m.cls_offset[size_t(cls) * 24];
    const double* a = off + 3 * m.tt.tri[t][0];
    const double* b = off + 3 * m.tt.tri[t][1];
    const double* c = off + 3 * m.tt.tri[t][2];
    const double x = b[1] * c[2] - b[2] * c[1];
    const double y = b[2] * c[0] - b[0] * c[2];
    const double z = b[0] * c[1] - b[1] * c[0];
    return std::fabs(a[0] * x + a[1] * y + a[2] * z) / 6.0;
}

inline void position(const HexMesh& m, long long tet, const double* bary, double* x) {
    const int c = int(tet / 12), t = int(tet % 12);
    const double* off = &m.cls_offset[size_t(m.cell_class[c]) * 24];
    for (int a = 0; a < 3; ++a) {
        x[a] = m.cc[3 * size_t(c) + a] + bary[0] * off[3 * m.tt.tri[t][0] + a] +
               bary[1] * off[3 * m.tt.tri[t][1] + a] + bary[2] * off[3 * m.tt.tri[t][2] + a];
    }
}

// `copies` topologically disjoint copies of one block mesh: a batched
// ensemble of independent cases in one store.  Cell, point and boundary-face
// indices of copy k are those of the single case plus k times the case's
// counts; geometry classes, patches and coordinates are shared (the copies
// overlap in space, which only the host-side locate/position calls see: they
// address copy 0).  Patch areas and face counts are totals over the copies.
inline HexMesh replicate_mesh(const HexMesh& one, int copies) {
    if (copies <= 1) return one;
    HexMesh m = one;
    const int nc = one.n_cells, np = one.n_points, ngp = one.n_grid_points;
    const int nbf = int(one.bfaces.size());
    m.n_cells = nc * copies;
    m.n_points = np * copies;
    m.n_grid_points = ngp * copies;
    auto raw = [copies](std::vector<double>& v) {
        const size_t n = v.size();
        v.resize(n * copies);
        for (int k = 1; k < copies; ++k) std::copy(v.begin(), v.begin() + n, v.begin() + k * n);
    };
    auto raw_i = [copies](std::vector<int>& v) {
        const size_t n = v.size();
        v.resize(n * copies);
        for (int k = 1; k < copies; ++k) std::copy(v.begin(), v.begin() + n, v.begin() + k * n);
    };
    auto shifted = [copies](const std::vector<int>& src, int step, bool keep_negative) {
        std::vector<int> v(src.size() * copies);
        for (int k = 0; k < copies; ++k)
            for (size_t i = 0; i < src.size(); ++i) {
                const int x = src[i];
                v[k * src.size() + i] = (keep_negative && x < 0) ? x : x + k * step;
            }
        return v;
    };
    raw(m.grid_pts);
    raw_i(m.cell_ijk);
    raw(m.cc);
    raw(m.vol);
    raw_i(m.cell_class);
    raw(m.lap_off);
    raw(m.lap_diag);
    raw(m.ip_weight);
    raw(m.vw_weight);
    m.cell_gpt = shifted(one.cell_gpt, ngp, false);
    m.cell_pt = shifted(one.cell_pt, np, false);
    m.nbr = shifted(one.nbr, nc, true);
    m.cell_bface = shifted(one.cell_bface, nbf, true);
    m.bfaces.clear();
    for (int k = 0; k < copies; ++k)
        for (BFace b : one.bfaces) {
            b.cell += k * nc;
            m.bfaces.push_back(b);
        }
    for (Patch& p : m.patches) {
        p.area *= copies;
        p.n_faces *= copies;
    }
    // CSR point interpolation: sources are cells (>= 0) or boundary faces (< 0)
    m.pi_start.assign(size_t(np) * copies + 1, 0);
    m.pi_src.clear();
    m.pi_w.clear();
    for (int k = 0; k < copies; ++k) {
        for (int p = 0; p < np; ++p) {
            m.pi_start[size_t(k) * np + p] = int(m.pi_src.size());
            for (int q = one.pi_start[p]; q < one.pi_start[p + 1]; ++q) {
                const int src = one.pi_src[q];
                m.pi_src.push_back(src >= 0 ? src + k * nc : -(-src - 1 + k * nbf) - 1);
                m.pi_w.push_back(one.pi_w[q]);
            }
        }
    }
    m.pi_start[size_t(np) * copies] = int(m.pi_src.size());
    // point -> cell-corner slots 9 c + 1 + corner
    m.pc_start.assign(size_t(np) * copies + 1, 0);
    m.pc_slot.clear();
    for (int k = 0; k < copies; ++k) {
        for (int p = 0; p < np; ++p) {
            m.pc_start[size_t(k) * np + p] = int(m.pc_slot.size());
            for (int q = one.pc_start[p]; q < one.pc_start[p + 1]; ++q) m.pc_slot.push_back(one.pc_slot[q] + 9 * k * nc);
        }
    }
    m.pc_start[size_t(np) * copies] = int(m.pc_slot.size());
    return m;
}

}  // namespace pg
