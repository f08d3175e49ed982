// Host-side mesh construction for the device layout.
//
// Topology derivation follows the reference reader's rule
// (src/MeshReader.cpp:317-456): faces are created while walking each
// cell's polygon edges in order; the first cell to visit an edge owns the
// face (cell_left) and fixes its node order, the second becomes cell_right.
// Reproducing that rule exactly is what makes face numbering, face
// orientation and every cell's face order identical to the reference, and
// with them the summation order of each cell residual.
#include "mesh_host.h"

#include <algorithm>
#include <cmath>
#include <map>
#include <numeric>
#include <queue>
#include <unordered_map>

namespace fvgb {

namespace {

[[noreturn]] void fail(int code, const std::string& msg) { throw MeshError{code, msg}; }

constexpr int kBadArg = 1;
constexpr int kBadMesh = 5;

inline uint64_t edge_key(int32_t a, int32_t b) {
    uint32_t lo = (uint32_t)std::min(a, b), hi = (uint32_t)std::max(a, b);
    return ((uint64_t)lo << 32) | hi;
}

bool segments_cross(double ax, double ay, double bx, double by, double cx, double cy, double dx, double dy) {
    auto side = [](double ox, double oy, double px, double py, double qx, double qy) {
        return (px - ox) * (qy - oy) - (py - oy) * (qx - ox);
    };
    double d1 = side(cx, cy, dx, dy, ax, ay), d2 = side(cx, cy, dx, dy, bx, by);
    double d3 = side(ax, ay, bx, by, cx, cy), d4 = side(ax, ay, bx, by, dx, dy);
    return ((d1 > 0 && d2 < 0) || (d1 < 0 && d2 > 0)) && ((d3 > 0 && d4 < 0) || (d3 < 0 && d4 > 0));
}

}  // namespace

// Face midpoint, length and unit normal (edge rotated -90 degrees):
// UnstructuredMesh::compute_geometry, include/UnstructuredMesh.h:89-105.
void HostMesh::compute_face_geometry() {
    fnx.resize(n_faces); fny.resize(n_faces); farea.resize(n_faces); fxm.resize(n_faces); fym.resize(n_faces);
    for (int32_t f = 0; f < n_faces; ++f) {
        double x1 = nx_[fn1[f]], y1 = ny_[fn1[f]], x2 = nx_[fn2[f]], y2 = ny_[fn2[f]];
        fxm[f] = 0.5 * (x1 + x2);
        fym[f] = 0.5 * (y1 + y2);
        double dx = x2 - x1, dy = y2 - y1;
        double a = std::sqrt(dx * dx + dy * dy);
        farea[f] = a;
        fnx[f] = dy / a;
        fny[f] = -dx / a;
    }
}

void build_from_polygons(HostMesh& m, int32_t n_nodes, const double* xy, int32_t n_cells, const int64_t* cell_off,
                         const int32_t* cell_nodes, int32_t n_bedges, const int32_t* bedge_nodes,
                         const int32_t* bedge_patch, int32_t n_patches) {
    if (n_nodes <= 0 || n_cells <= 0 || !xy || !cell_off || !cell_nodes || n_bedges < 0 || n_patches < 0)
        fail(kBadArg, "mesh: empty or null input");
    if (n_bedges > 0 && (!bedge_nodes || !bedge_patch)) fail(kBadArg, "mesh: null boundary arrays");
    m.n_nodes = n_nodes; m.n_cells = n_cells; m.n_patches = n_patches;
    m.nx_.resize(n_nodes); m.ny_.resize(n_nodes);
    for (int32_t i = 0; i < n_nodes; ++i) {
        m.nx_[i] = xy[2 * i]; m.ny_[i] = xy[2 * i + 1];
        if (!std::isfinite(m.nx_[i]) || !std::isfinite(m.ny_[i]))
            fail(kBadMesh, "mesh: node " + std::to_string(i) + " has a non-finite coordinate");
    }
    if (cell_off[0] != 0) fail(kBadArg, "mesh: cell_off[0] != 0");
    m.cnode_off.assign(cell_off, cell_off + n_cells + 1);
    m.cnodes.assign(cell_nodes, cell_nodes + cell_off[n_cells]);
    std::unordered_map<uint64_t, int32_t> edge_to_face;
    edge_to_face.reserve((size_t)(cell_off[n_cells] * 0.6) + 16);
    m.cf_off.assign(n_cells + 1, 0);
    m.cf.reserve((size_t)cell_off[n_cells]);
    m.vol.resize(n_cells); m.cx.resize(n_cells); m.cy.resize(n_cells);
    for (int32_t c = 0; c < n_cells; ++c) {
        int64_t lo = cell_off[c], hi = cell_off[c + 1];
        int32_t k = (int32_t)(hi - lo);
        if (k < 3) fail(kBadMesh, "mesh: cell " + std::to_string(c) + " has fewer than 3 vertices");
        const int32_t* ids = cell_nodes + lo;
        for (int32_t e = 0; e < k; ++e) {
            int32_t a = ids[e], b = ids[(e + 1) % k];
            if (a < 0 || a >= n_nodes || b < 0 || b >= n_nodes)
                fail(kBadMesh, "mesh: cell " + std::to_string(c) + " references an out-of-range node");
            auto it = edge_to_face.find(edge_key(a, b));
            if (it == edge_to_face.end()) {
                int32_t f = (int32_t)m.fn1.size();
                m.fn1.push_back(a); m.fn2.push_back(b); m.fl.push_back(c); m.fr.push_back(-1);
                m.fpatch.push_back(-1);
                edge_to_face.emplace(edge_key(a, b), f);
                m.cf.push_back(f);
            } else {
                int32_t f = it->second;
                if (m.fr[f] != -1) fail(kBadMesh, "mesh: edge shared by more than two cells");
                m.fr[f] = c;
                m.cf.push_back(f);
            }
        }
        m.cf_off[c + 1] = (int32_t)m.cf.size();
        // Shoelace area and centroid with the signed area
        // (src/MeshReader.cpp:32-41, :56-76).
        double area = 0.0;
        for (int32_t i = 0; i < k; ++i) {
            int32_t p0 = ids[i], p1 = ids[(i + 1) % k];
            area += m.nx_[p0] * m.ny_[p1] - m.nx_[p1] * m.ny_[p0];
        }
        area = 0.5 * area;
        double sx = 0.0, sy = 0.0;
        for (int32_t i = 0; i < k; ++i) {
            int32_t p0 = ids[i], p1 = ids[(i + 1) % k];
            double cross = m.nx_[p0] * m.ny_[p1] - m.nx_[p1] * m.ny_[p0];
            sx += (m.nx_[p0] + m.nx_[p1]) * cross;
            sy += (m.ny_[p0] + m.ny_[p1]) * cross;
        }
        sx /= (6.0 * area);
        sy /= (6.0 * area);
        if (!std::isfinite(area) || area <= 0.0)
            fail(kBadMesh, "mesh: cell " + std::to_string(c) + " has non-positive signed area (clockwise or degenerate)");
        for (int32_t i = 0; i < k; ++i)
            for (int32_t j = i + 2; j < k; ++j) {
                if (i == 0 && j == k - 1) continue;
                int32_t a0 = ids[i], a1 = ids[(i + 1) % k], b0 = ids[j], b1 = ids[(j + 1) % k];
                if (segments_cross(m.nx_[a0], m.ny_[a0], m.nx_[a1], m.ny_[a1], m.nx_[b0], m.ny_[b0], m.nx_[b1],
                                   m.ny_[b1]))
                    fail(kBadMesh, "mesh: cell " + std::to_string(c) + " is self-intersecting");
            }
        m.vol[c] = std::fabs(area);
        m.cx[c] = sx;
        m.cy[c] = sy;
    }
    m.n_faces = (int32_t)m.fn1.size();
    for (int32_t i = 0; i < n_bedges; ++i) {
        int32_t a = bedge_nodes[2 * i], b = bedge_nodes[2 * i + 1], p = bedge_patch[i];
        if (p < 0 || p >= n_patches) fail(kBadArg, "mesh: boundary edge patch index out of range");
        auto it = edge_to_face.find(edge_key(a, b));
        if (it == edge_to_face.end()) continue;  // matches no cell edge: ignored, as in the reference
        m.fpatch[it->second] = p;
    }
    int64_t untagged = 0;
    for (int32_t f = 0; f < m.n_faces; ++f)
        if (m.fr[f] == -1 && m.fpatch[f] == -1) ++untagged;
    if (untagged) fail(kBadMesh, "mesh: " + std::to_string(untagged) + " boundary faces have no patch");
    m.compute_face_geometry();
    for (int32_t f = 0; f < m.n_faces; ++f)
        if (!(m.farea[f] > 0.0) || !std::isfinite(m.farea[f]))
            fail(kBadMesh, "mesh: face " + std::to_string(f) + " has zero or non-finite length");
}

void build_from_faces(HostMesh& m, int32_t n_nodes, const double* xy, int32_t n_faces, const int32_t* face_nodes,
                      const int32_t* face_cells, const int32_t* face_patch, int32_t n_cells,
                      const int32_t* cell_face_off, const int32_t* cell_faces, const double* cell_geom,
                      int32_t n_patches) {
    if (n_nodes <= 0 || n_cells <= 0 || n_faces <= 0 || !xy || !face_nodes || !face_cells || !face_patch ||
        !cell_face_off || !cell_faces || !cell_geom)
        fail(kBadArg, "mesh: empty or null input");
    m.n_nodes = n_nodes; m.n_cells = n_cells; m.n_faces = n_faces; m.n_patches = n_patches;
    m.nx_.resize(n_nodes); m.ny_.resize(n_nodes);
    for (int32_t i = 0; i < n_nodes; ++i) { m.nx_[i] = xy[2 * i]; m.ny_[i] = xy[2 * i + 1]; }
    m.fn1.resize(n_faces); m.fn2.resize(n_faces); m.fl.resize(n_faces); m.fr.resize(n_faces);
    m.fpatch.resize(n_faces);
    for (int32_t f = 0; f < n_faces; ++f) {
        m.fn1[f] = face_nodes[2 * f]; m.fn2[f] = face_nodes[2 * f + 1];
        m.fl[f] = face_cells[2 * f]; m.fr[f] = face_cells[2 * f + 1];
        m.fpatch[f] = face_patch[f];
        if (m.fn1[f] < 0 || m.fn1[f] >= n_nodes || m.fn2[f] < 0 || m.fn2[f] >= n_nodes)
            fail(kBadMesh, "mesh: face node index out of range");
        if (m.fl[f] < 0 || m.fl[f] >= n_cells || m.fr[f] < -1 || m.fr[f] >= n_cells)
            fail(kBadMesh, "mesh: face cell index out of range");
        if (m.fr[f] == -1 && (m.fpatch[f] < 0 || m.fpatch[f] >= n_patches))
            fail(kBadMesh, "mesh: boundary face " + std::to_string(f) + " has no valid patch");
    }
    m.cf_off.assign(cell_face_off, cell_face_off + n_cells + 1);
    if (m.cf_off[0] != 0) fail(kBadArg, "mesh: cell_face_off[0] != 0");
    m.cf.assign(cell_faces, cell_faces + m.cf_off[n_cells]);
    for (int32_t c = 0; c < n_cells; ++c)
        for (int32_t e = m.cf_off[c]; e < m.cf_off[c + 1]; ++e) {
            int32_t f = m.cf[e];
            if (f < 0 || f >= n_faces || (m.fl[f] != c && m.fr[f] != c))
                fail(kBadMesh, "mesh: cell " + std::to_string(c) + " lists a face it does not bound");
        }
    m.vol.resize(n_cells); m.cx.resize(n_cells); m.cy.resize(n_cells);
    for (int32_t c = 0; c < n_cells; ++c) {
        m.vol[c] = cell_geom[3 * c]; m.cx[c] = cell_geom[3 * c + 1]; m.cy[c] = cell_geom[3 * c + 2];
        if (!(m.vol[c] > 0.0) || !std::isfinite(m.vol[c])) fail(kBadMesh, "mesh: non-positive cell volume");
    }
    m.compute_face_geometry();
    for (int32_t f = 0; f < n_faces; ++f)
        if (!(m.farea[f] > 0.0) || !std::isfinite(m.farea[f])) fail(kBadMesh, "mesh: zero-length face");
}

namespace {

uint64_t interleave32(uint32_t x, uint32_t y) {
    auto spread = [](uint64_t v) {
        v &= 0xffffffffull;
        v = (v | (v << 16)) & 0x0000ffff0000ffffull;
        v = (v | (v << 8)) & 0x00ff00ff00ff00ffull;
        v = (v | (v << 4)) & 0x0f0f0f0f0f0f0f0full;
        v = (v | (v << 2)) & 0x3333333333333333ull;
        v = (v | (v << 1)) & 0x5555555555555555ull;
        return v;
    };
    return spread(x) | (spread(y) << 1);
}

// Morton (Z-order) of the centroids of cells [c0, c1).
std::vector<int32_t> morton_order(const HostMesh& m, int32_t c0, int32_t c1) {
    double xmin = *std::min_element(m.cx.begin() + c0, m.cx.begin() + c1);
    double xmax = *std::max_element(m.cx.begin() + c0, m.cx.begin() + c1);
    double ymin = *std::min_element(m.cy.begin() + c0, m.cy.begin() + c1);
    double ymax = *std::max_element(m.cy.begin() + c0, m.cy.begin() + c1);
    double span = std::max(xmax - xmin, ymax - ymin);
    if (!(span > 0.0)) span = 1.0;
    double s = 4294967295.0 / span;
    std::vector<std::pair<uint64_t, int32_t>> key(c1 - c0);
    for (int32_t c = c0; c < c1; ++c) {
        uint32_t qx = (uint32_t)std::min(4294967295.0, (m.cx[c] - xmin) * s);
        uint32_t qy = (uint32_t)std::min(4294967295.0, (m.cy[c] - ymin) * s);
        key[c - c0] = {interleave32(qx, qy), c};
    }
    std::sort(key.begin(), key.end());
    std::vector<int32_t> perm(c1 - c0);
    for (int32_t i = 0; i < c1 - c0; ++i) perm[i] = key[i].second;
    return perm;
}

// Reverse Cuthill-McKee over the cell adjacency graph (internal faces).
std::vector<int32_t> rcm_order(const HostMesh& m) {
    int32_t n = m.n_cells;
    std::vector<int32_t> deg(n, 0);
    for (int32_t c = 0; c < n; ++c)
        for (int32_t e = m.cf_off[c]; e < m.cf_off[c + 1]; ++e)
            if (m.fr[m.cf[e]] >= 0) ++deg[c];
    auto neighbors = [&](int32_t c, std::vector<int32_t>& out) {
        out.clear();
        for (int32_t e = m.cf_off[c]; e < m.cf_off[c + 1]; ++e) {
            int32_t f = m.cf[e];
            if (m.fr[f] < 0) continue;
            out.push_back(m.fl[f] == c ? m.fr[f] : m.fl[f]);
        }
        std::sort(out.begin(), out.end(), [&](int32_t a, int32_t b) { return deg[a] < deg[b] || (deg[a] == deg[b] && a < b); });
    };
    std::vector<int32_t> order;
    order.reserve(n);
    std::vector<char> seen(n, 0);
    std::vector<int32_t> nb;
    auto bfs = [&](int32_t start, std::vector<int32_t>* out) {
        // Returns the last node reached; appends visit order to *out if given.
        std::vector<int32_t> local;
        std::queue<int32_t> q;
        std::vector<char> s2;
        std::vector<char>& mark = out ? seen : (s2 = seen, s2);
        q.push(start); mark[start] = 1;
        int32_t last = start;
        while (!q.empty()) {
            int32_t c = q.front(); q.pop();
            last = c;
            if (out) out->push_back(c);
            neighbors(c, nb);
            for (int32_t o : nb) if (!mark[o]) { mark[o] = 1; q.push(o); }
        }
        return last;
    };
    for (int32_t c0 = 0; c0 < n; ++c0) {
        if (seen[c0]) continue;
        int32_t far1 = bfs(c0, nullptr);
        int32_t far2 = bfs(far1, nullptr);
        bfs(far2, &order);
    }
    std::reverse(order.begin(), order.end());
    return order;
}

}  // namespace

void HostMesh::build_device_layout(int reorder) {
    // Groups (batched meshes: one per instance) stay contiguous and in
    // order; the space-filling-curve order applies within each group.
    std::vector<int32_t> groups = group_off;
    if (groups.empty()) groups = {0, n_cells};
    if (reorder == 2 && groups.size() == 2) perm = rcm_order(*this);
    else {
        perm.clear();
        perm.reserve(n_cells);
        for (size_t g = 0; g + 1 < groups.size(); ++g) {
            if (reorder == 0) {
                for (int32_t c = groups[g]; c < groups[g + 1]; ++c) perm.push_back(c);
            } else {
                std::vector<int32_t> p = morton_order(*this, groups[g], groups[g + 1]);
                perm.insert(perm.end(), p.begin(), p.end());
            }
        }
    }
    if (reorder != 0) {
        // Within each tile of 256 consecutive cells (one thread block) of a
        // group, order the cells by face count: each warp then runs its
        // per-face loops with one trip count, and a warp's instructions are
        // issued once for all its cells.  Locality is kept at tile granularity.
        const int32_t tile = 256;
        for (size_t g = 0; g + 1 < groups.size(); ++g)
            for (int32_t t0 = groups[g]; t0 < groups[g + 1]; t0 += tile) {
                const int32_t t1 = std::min(groups[g + 1], t0 + tile);
                std::stable_sort(perm.begin() + t0, perm.begin() + t1, [&](int32_t a, int32_t b) {
                    return cf_off[a + 1] - cf_off[a] < cf_off[b + 1] - cf_off[b];
                });
            }
    }
    iperm.assign(n_cells, 0);
    for (int32_t i = 0; i < n_cells; ++i) iperm[perm[i]] = i;

    // Faces: internal first sorted by (owner, neighbour) in device order,
    // then boundary faces sorted by (patch, owner).
    fperm.resize(n_faces);
    std::iota(fperm.begin(), fperm.end(), 0);
    std::sort(fperm.begin(), fperm.end(), [&](int32_t a, int32_t b) {
        bool ba = fr[a] < 0, bb = fr[b] < 0;
        if (ba != bb) return !ba;
        if (ba) {
            if (fpatch[a] != fpatch[b]) return fpatch[a] < fpatch[b];
            return iperm[fl[a]] < iperm[fl[b]];
        }
        if (iperm[fl[a]] != iperm[fl[b]]) return iperm[fl[a]] < iperm[fl[b]];
        return iperm[fr[a]] < iperm[fr[b]];
    });
    ifperm.assign(n_faces, 0);
    n_int_faces = 0;
    for (int32_t i = 0; i < n_faces; ++i) {
        ifperm[fperm[i]] = i;
        if (fr[fperm[i]] >= 0) ++n_int_faces;
    }
    d_fl.resize(n_faces); d_fr.resize(n_faces); d_fpatch.resize(n_faces);
    d_fgeom.resize(4 * (size_t)n_faces); d_fmid.resize(2 * (size_t)n_faces);
    for (int32_t i = 0; i < n_faces; ++i) {
        int32_t f = fperm[i];
        d_fl[i] = iperm[fl[f]];
        d_fr[i] = fr[f] >= 0 ? iperm[fr[f]] : -1;
        d_fpatch[i] = fpatch[f];
        d_fgeom[4 * i + 0] = fnx[f];
        d_fgeom[4 * i + 1] = fny[f];
        d_fgeom[4 * i + 2] = farea[f];
        // Characteristic length of the CFL estimate (src/EulerFVMSolver.cpp:151-156).
        d_fgeom[4 * i + 3] = fr[f] >= 0 ? std::min(vol[fl[f]], vol[fr[f]]) / farea[f] : vol[fl[f]] / farea[f];
        d_fmid[2 * i] = fxm[f];
        d_fmid[2 * i + 1] = fym[f];
    }
    d_cf_off.assign(n_cells + 1, 0);
    d_cf.resize(cf.size());
    d_vol.resize(n_cells); d_cxy.resize(2 * (size_t)n_cells);
    int32_t pos = 0;
    for (int32_t i = 0; i < n_cells; ++i) {
        int32_t c = perm[i];
        d_vol[i] = vol[c];
        d_cxy[2 * i] = cx[c];
        d_cxy[2 * i + 1] = cy[c];
        for (int32_t e = cf_off[c]; e < cf_off[c + 1]; ++e) {
            int32_t f = cf[e];
            d_cf[pos++] = (ifperm[f] << 1) | (fl[f] == c ? 1 : 0);
        }
        d_cf_off[i + 1] = pos;
    }
}

// Per-entry and per-face geometry of the second-order scheme (device order).
//  LSQ: the weighted least-squares gradient of GradientCalculator
//  (src/GradientReconstruction.cpp:45-80, :124-148; weights 1/d^2 over face
//  neighbours, boundary-face midpoints standing in for missing neighbours)
//  is linear in the differences phi_j - phi_c, so the inverse normal matrix
//  is folded into one weight pair per entry: grad = sum_j (a_j, b_j) dphi_j.
//  GG: Green-Gauss with inverse-distance face values (:89-118).
void HostMesh::build_o2_geometry() {
    size_t E = d_cf.size();
    d_cnb.resize(E);
    d_lsq.resize(2 * E);
    d_lsq_sum.assign(2 * (size_t)n_cells, 0.0);
    d_gg.resize(4 * E);
    d_erf.resize(2 * E);
    d_frf.assign(4 * (size_t)n_faces, 0.0);
    d_h.resize(n_cells);
    for (int32_t i = 0; i < n_cells; ++i) {
        int32_t c = perm[i];
        double xc = cx[c], yc = cy[c];
        d_h[i] = std::sqrt(vol[c]);
        int32_t e0 = d_cf_off[i], e1 = d_cf_off[i + 1];
        double m00 = 0.0, m01 = 0.0, m11 = 0.0;
        for (int32_t e = e0; e < e1; ++e) {
            int32_t f = fperm[d_cf[e] >> 1];
            double px, py;
            if (fr[f] < 0) { px = fxm[f]; py = fym[f]; }
            else {
                int32_t nb = fl[f] == c ? fr[f] : fl[f];
                px = cx[nb]; py = cy[nb];
            }
            double dx = px - xc, dy = py - yc;
            double w = 1.0 / (dx * dx + dy * dy);
            m00 += w * dx * dx; m01 += w * dx * dy; m11 += w * dy * dy;
        }
        double det = m00 * m11 - m01 * m01;
        double i00 = m11 / det, i01 = -m01 / det, i11 = m00 / det;
        for (int32_t e = e0; e < e1; ++e) {
            int32_t fd = d_cf[e] >> 1;
            int32_t f = fperm[fd];
            bool owner = fl[f] == c;
            double px, py;
            if (fr[f] < 0) {
                px = fxm[f]; py = fym[f];
                d_cnb[e] = -1 - fd;
            } else {
                int32_t nb = owner ? fr[f] : fl[f];
                px = cx[nb]; py = cy[nb];
                d_cnb[e] = iperm[nb];
            }
            double dx = px - xc, dy = py - yc;
            double w = 1.0 / (dx * dx + dy * dy);
            d_lsq[2 * e] = i00 * (w * dx) + i01 * (w * dy);
            d_lsq[2 * e + 1] = i01 * (w * dx) + i11 * (w * dy);
            d_lsq_sum[2 * i] += d_lsq[2 * e];
            d_lsq_sum[2 * i + 1] += d_lsq[2 * e + 1];
            double sgn = owner ? 1.0 : -1.0;
            d_gg[4 * e] = sgn * fnx[f] * farea[f] / vol[c];
            d_gg[4 * e + 1] = sgn * fny[f] * farea[f] / vol[c];
            if (fr[f] < 0) d_gg[4 * e + 2] = 0.0;
            else {
                double d_c = std::hypot(xc - fxm[f], yc - fym[f]);
                double d_o = std::hypot(px - fxm[f], py - fym[f]);
                d_gg[4 * e + 2] = d_o / (d_c + d_o);
            }
            d_gg[4 * e + 3] = 0.0;
            d_erf[2 * e] = fxm[f] - xc;
            d_erf[2 * e + 1] = fym[f] - yc;
        }
    }
    for (int32_t i = 0; i < n_faces; ++i) {
        int32_t f = fperm[i];
        d_frf[4 * i] = fxm[f] - cx[fl[f]];
        d_frf[4 * i + 1] = fym[f] - cy[fl[f]];
        if (fr[f] >= 0) {
            d_frf[4 * i + 2] = fxm[f] - cx[fr[f]];
            d_frf[4 * i + 3] = fym[f] - cy[fr[f]];
        }
    }
}

}  // namespace fvgb

namespace fvgb {

// GradientCalculator ctor (src/GradientReconstruction.cpp:45-80): per-cell
// inverse normal matrix, and the per-entry terms compute() needs
// (:83-150); face_normal_geometry / face_gradient (:25-40, :153-183).
void build_grad_geom(const HostMesh& m, HostGradGeom& g) {
    const int32_t N = m.n_cells, F = m.n_faces;
    const size_t E = m.d_cf.size();
    g.nb.resize(E);
    g.lsq_w.resize(2 * E);
    g.gg.resize(4 * E);
    g.lsq_inv.resize(3 * (size_t)N);
    g.fgrad.assign(8 * (size_t)F, 0.0);
    for (int32_t i = 0; i < N; ++i) {
        const int32_t c = m.perm[i];
        const double xc = m.cx[c], yc = m.cy[c];
        double m00 = 0.0, m01 = 0.0, m11 = 0.0;
        for (int32_t e = m.d_cf_off[i]; e < m.d_cf_off[i + 1]; ++e) {
            const int32_t fd = m.d_cf[e] >> 1;
            const int32_t f = m.fperm[fd];
            double nx, ny;
            if (m.fr[f] == -1) {
                nx = m.fxm[f];
                ny = m.fym[f];
                g.nb[e] = -1 - fd;
            } else {
                const int32_t nbr = (m.fl[f] == c) ? m.fr[f] : m.fl[f];
                nx = m.cx[nbr];
                ny = m.cy[nbr];
                g.nb[e] = m.iperm[nbr];
            }
            const double dx = nx - xc;
            const double dy = ny - yc;
            const double w = 1.0 / (dx * dx + dy * dy);
            m00 += w * dx * dx;
            m01 += w * dx * dy;
            m11 += w * dy * dy;
            g.lsq_w[2 * e] = w * dx;
            g.lsq_w[2 * e + 1] = w * dy;
            // Green-Gauss: outward normal of this cell, face length and the
            // inverse-distance weight of the owning side.
            const bool owner = m.fl[f] == c;
            g.gg[4 * e] = owner ? m.fnx[f] : -m.fnx[f];
            g.gg[4 * e + 1] = owner ? m.fny[f] : -m.fny[f];
            g.gg[4 * e + 2] = m.farea[f];
            if (m.fr[f] == -1) {
                g.gg[4 * e + 3] = 0.0;
            } else {
                const int32_t other = owner ? m.fr[f] : m.fl[f];
                const double d_c = std::hypot(xc - m.fxm[f], yc - m.fym[f]);
                const double d_o = std::hypot(m.cx[other] - m.fxm[f], m.cy[other] - m.fym[f]);
                g.gg[4 * e + 3] = d_o / (d_c + d_o);
            }
        }
        const double det = m00 * m11 - m01 * m01;
        g.lsq_inv[3 * (size_t)i] = m11 / det;
        g.lsq_inv[3 * (size_t)i + 1] = -m01 / det;
        g.lsq_inv[3 * (size_t)i + 2] = m00 / det;
    }
    for (int32_t i = 0; i < F; ++i) {
        const int32_t f = m.fperm[i];
        const int32_t cl = m.fl[f];
        const bool bnd = m.fr[f] == -1;
        const double xR = bnd ? m.fxm[f] : m.cx[m.fr[f]];
        const double yR = bnd ? m.fym[f] : m.cy[m.fr[f]];
        const double dx = xR - m.cx[cl];
        const double dy = yR - m.cy[cl];
        const double dist = std::hypot(dx, dy);
        const double dhx = dx / dist, dhy = dy / dist;
        const double cos_theta = m.fnx[f] * dhx + m.fny[f] * dhy;
        double* o = &g.fgrad[8 * (size_t)i];
        o[0] = dist;
        o[1] = cos_theta;
        o[2] = m.fnx[f] - dhx / cos_theta;
        o[3] = m.fny[f] - dhy / cos_theta;
        if (!bnd) {
            const double d_L = std::hypot(m.cx[cl] - m.fxm[f], m.cy[cl] - m.fym[f]);
            const double d_R = std::hypot(xR - m.fxm[f], yR - m.fym[f]);
            o[4] = d_R / (d_L + d_R);
        }
        o[5] = dist * cos_theta;
        o[6] = m.fnx[f];
        o[7] = m.fny[f];
    }
}

void concat_meshes(const std::vector<const HostMesh*>& parts, HostMesh& out) {
    if (parts.empty()) throw MeshError{1, "batch: no meshes"};
    out = HostMesh{};
    out.n_patches = parts[0]->n_patches;
    out.group_off.push_back(0);
    int32_t node0 = 0, cell0 = 0, face0 = 0;
    for (const HostMesh* p : parts) {
        if (p->n_patches != out.n_patches) throw MeshError{1, "batch: meshes have different patch counts"};
        out.nx_.insert(out.nx_.end(), p->nx_.begin(), p->nx_.end());
        out.ny_.insert(out.ny_.end(), p->ny_.begin(), p->ny_.end());
        for (int32_t f = 0; f < p->n_faces; ++f) {
            out.fn1.push_back(p->fn1[f] + node0);
            out.fn2.push_back(p->fn2[f] + node0);
            out.fl.push_back(p->fl[f] + cell0);
            out.fr.push_back(p->fr[f] >= 0 ? p->fr[f] + cell0 : -1);
            out.fpatch.push_back(p->fpatch[f]);
        }
        out.fnx.insert(out.fnx.end(), p->fnx.begin(), p->fnx.end());
        out.fny.insert(out.fny.end(), p->fny.begin(), p->fny.end());
        out.farea.insert(out.farea.end(), p->farea.begin(), p->farea.end());
        out.fxm.insert(out.fxm.end(), p->fxm.begin(), p->fxm.end());
        out.fym.insert(out.fym.end(), p->fym.begin(), p->fym.end());
        if (out.cf_off.empty()) out.cf_off.push_back(0);
        for (int32_t c = 0; c < p->n_cells; ++c) {
            for (int32_t e = p->cf_off[c]; e < p->cf_off[c + 1]; ++e) out.cf.push_back(p->cf[e] + face0);
            out.cf_off.push_back((int32_t)out.cf.size());
        }
        out.vol.insert(out.vol.end(), p->vol.begin(), p->vol.end());
        out.cx.insert(out.cx.end(), p->cx.begin(), p->cx.end());
        out.cy.insert(out.cy.end(), p->cy.begin(), p->cy.end());
        node0 += p->n_nodes;
        cell0 += p->n_cells;
        face0 += p->n_faces;
        out.group_off.push_back(cell0);
    }
    out.n_nodes = node0;
    out.n_cells = cell0;
    out.n_faces = face0;
}

// Agglomeration: seeds in the fine mesh's device order (space-filling
// curve); each seed takes its unassigned face neighbours by decreasing
// shared face length up to four cells, then the unassigned neighbours of
// those; leftover single cells join the neighbouring agglomerate they share
// the longest face with.
void agglomerate(const HostMesh& f, std::vector<int32_t>& agg, HostMesh& c) {
    const int N = f.n_cells;
    agg.assign(N, -1);
    std::vector<int32_t> size;
    auto neighbours = [&](int cell, std::vector<std::pair<double, int>>& out) {
        out.clear();
        for (int k = f.cf_off[cell]; k < f.cf_off[cell + 1]; ++k) {
            const int fc = f.cf[k];
            const int nb = f.fl[fc] == cell ? f.fr[fc] : f.fl[fc];
            if (nb >= 0) out.push_back({f.farea[fc], nb});
        }
        std::sort(out.begin(), out.end(), [](const std::pair<double, int>& a, const std::pair<double, int>& b) {
            return a.first > b.first || (a.first == b.first && a.second < b.second);
        });
    };
    std::vector<std::pair<double, int>> nb1, nb2;
    const int32_t* order = f.perm.empty() ? nullptr : f.perm.data();
    for (int ii = 0; ii < N; ++ii) {
        const int seed = order ? order[ii] : ii;
        if (agg[seed] >= 0) continue;
        const int id = (int)size.size();
        std::vector<int> mem = {seed};
        agg[seed] = id;
        neighbours(seed, nb1);
        for (auto& q : nb1)
            if ((int)mem.size() < 4 && agg[q.second] < 0) { agg[q.second] = id; mem.push_back(q.second); }
        for (size_t m = 1; m < mem.size() && (int)mem.size() < 4; ++m) {
            neighbours(mem[m], nb2);
            for (auto& q : nb2)
                if ((int)mem.size() < 4 && agg[q.second] < 0) { agg[q.second] = id; mem.push_back(q.second); }
        }
        size.push_back((int)mem.size());
    }
    // merge singletons into the neighbour agglomerate across their longest face
    for (int cell = 0; cell < N; ++cell) {
        const int id = agg[cell];
        if (size[id] != 1) continue;
        neighbours(cell, nb1);
        for (auto& q : nb1) {
            const int t = agg[q.second];
            if (t != id && size[t] < 6) {
                agg[cell] = t;
                size[t] += 1;
                size[id] = 0;
                break;
            }
        }
    }
    // compact ids
    std::vector<int32_t> remap(size.size(), -1);
    int nc = 0;
    for (int cell = 0; cell < N; ++cell)
        if (remap[agg[cell]] < 0) remap[agg[cell]] = nc++;
    for (int cell = 0; cell < N; ++cell) agg[cell] = remap[agg[cell]];
    c = HostMesh{};
    c.n_cells = nc;
    // batched meshes: agglomerates never cross instances (no faces join
    // them) and the ids follow the cell order, so each instance keeps a
    // contiguous range
    if (f.group_off.size() >= 2) {
        const size_t ni = f.group_off.size() - 1;
        std::vector<int32_t> go(ni + 1, nc);
        for (size_t i = 0; i < ni; ++i) go[i] = f.group_off[i] < N ? agg[f.group_off[i]] : nc;
        c.group_off.assign(go.begin(), go.end());
    }
    // coarse cells

    c.n_patches = f.n_patches;
    c.vol.assign(nc, 0.0);
    c.cx.assign(nc, 0.0);
    c.cy.assign(nc, 0.0);
    for (int cell = 0; cell < N; ++cell) {
        const int a = agg[cell];
        c.vol[a] += f.vol[cell];
        c.cx[a] += f.vol[cell] * f.cx[cell];
        c.cy[a] += f.vol[cell] * f.cy[cell];
    }
    for (int a = 0; a < nc; ++a) { c.cx[a] /= c.vol[a]; c.cy[a] /= c.vol[a]; }
    // coarse faces: (owner, neighbour or -1-patch) -> accumulated n A, A, x A
    std::map<std::pair<int, int>, int> key;
    std::vector<double> sx, sy, sa, smx, smy;
    for (int fc = 0; fc < f.n_faces; ++fc) {
        const int A = agg[f.fl[fc]];
        const int B = f.fr[fc] >= 0 ? agg[f.fr[fc]] : -1;
        if (B == A) continue;
        int o, n;
        double sgn = 1.0;
        if (B >= 0) {
            o = std::min(A, B);
            n = std::max(A, B);
            if (o != A) sgn = -1.0;
        } else {
            o = A;
            n = -1 - f.fpatch[fc];
        }
        auto it = key.find({o, n});
        int k;
        if (it == key.end()) {
            k = (int)sx.size();
            key.emplace(std::make_pair(o, n), k);
            sx.push_back(0.0); sy.push_back(0.0); sa.push_back(0.0); smx.push_back(0.0); smy.push_back(0.0);
            c.fl.push_back(o);
            c.fr.push_back(n >= 0 ? n : -1);
            c.fpatch.push_back(n >= 0 ? -1 : f.fpatch[fc]);
        } else {
            k = it->second;
        }
        sx[k] += sgn * f.fnx[fc] * f.farea[fc];
        sy[k] += sgn * f.fny[fc] * f.farea[fc];
        sa[k] += f.farea[fc];
        smx[k] += f.farea[fc] * f.fxm[fc];
        smy[k] += f.farea[fc] * f.fym[fc];
    }
    const int nf = (int)sx.size();
    c.n_faces = nf;
    c.fnx.resize(nf); c.fny.resize(nf); c.farea.resize(nf); c.fxm.resize(nf); c.fym.resize(nf);
    c.fn1.assign(nf, 0); c.fn2.assign(nf, 0);
    for (int k = 0; k < nf; ++k) {
        // merged faces whose normals cancel (|sum n A| = 0) carry no flux
        const double len = std::max(std::sqrt(sx[k] * sx[k] + sy[k] * sy[k]), 1e-300);
        c.farea[k] = len;
        c.fnx[k] = sx[k] / len;
        c.fny[k] = sy[k] / len;
        c.fxm[k] = smx[k] / sa[k];
        c.fym[k] = smy[k] / sa[k];
    }
    // cell -> faces
    std::vector<std::vector<int>> cf(nc);
    for (int k = 0; k < nf; ++k) {
        cf[c.fl[k]].push_back(k);
        if (c.fr[k] >= 0) cf[c.fr[k]].push_back(k);
    }
    c.cf_off.assign(nc + 1, 0);
    for (int a = 0; a < nc; ++a) c.cf_off[a + 1] = c.cf_off[a] + (int)cf[a].size();
    c.cf.reserve(c.cf_off[nc]);
    for (int a = 0; a < nc; ++a) c.cf.insert(c.cf.end(), cf[a].begin(), cf[a].end());
}

}  // namespace fvgb
