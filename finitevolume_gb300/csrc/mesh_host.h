// Host-side mesh: topology derivation, geometry, validation and the
// reordered structure-of-arrays layout that the device kernels read.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace fvgb {

struct MeshError {
    int code;
    std::string msg;
};

// Mesh in reference numbering (the fields of include/UnstructuredMesh.h:20-106
// as plain arrays), plus the device-order layout derived from it.
struct HostMesh {
    // --- reference numbering ---------------------------------------------
    int32_t n_nodes = 0, n_cells = 0, n_faces = 0, n_patches = 0;
    std::vector<double> nx_, ny_;                // node coordinates
    std::vector<int32_t> fn1, fn2, fl, fr, fpatch;
    std::vector<double> fnx, fny, farea, fxm, fym;
    std::vector<int32_t> cf_off, cf;              // cell -> faces, reference order
    std::vector<double> vol, cx, cy;
    // cell polygons (CCW node lists) when the mesh was built from them;
    // empty for meshes given as faces plus cell geometry
    std::vector<int64_t> cnode_off;
    std::vector<int32_t> cnodes;

    // --- device order (perm[new] = reference cell, fperm[new] = ref face) --
    std::vector<int32_t> perm, iperm, fperm, ifperm;
    int32_t n_int_faces = 0;                     // faces [0, n_int) are internal
    std::vector<int32_t> group_off;              // batched meshes: instance cell ranges (else empty)
    // SoA arrays in device order
    std::vector<int32_t> d_fl, d_fr, d_fpatch;   // right = -1 on boundary faces
    std::vector<double> d_fgeom;                 // [4F] nx, ny, area, dt-length
    std::vector<double> d_fmid;                  // [2F] x_mid, y_mid
    std::vector<int32_t> d_cf_off, d_cf;         // entries: face<<1 | (cell is owner)
    std::vector<double> d_vol, d_cxy;            // [N], [2N]

    // Second-order geometry, device order (built by build_o2_geometry).
    std::vector<int32_t> d_cnb;                  // per entry: neighbour cell, or -1-face for boundary
    std::vector<double> d_lsq;                   // per entry [2]: LSQ weights folded with the inverse matrix
    std::vector<double> d_lsq_sum;               // per cell [2]: sums of those weights
    std::vector<double> d_gg;                    // per entry [4]: Green-Gauss s*A*nx/V, s*A*ny/V, owner weight, 0
    std::vector<double> d_erf;                   // per entry [2]: face midpoint - cell centroid
    std::vector<double> d_frf;                   // per face [4]: x_f - x_L, x_f - x_R (R: zero on boundary)
    std::vector<double> d_h;                     // per cell: sqrt(volume) (limiter length scale)

    void compute_face_geometry();                // UnstructuredMesh::compute_geometry
    void build_device_layout(int reorder);
    void build_o2_geometry();
};

// Geometry of the reference's GradientCalculator and face_gradient
// (src/GradientReconstruction.cpp:12-200), device order, computed on the
// host with the reference's own expressions (so strict device code that
// consumes it reproduces the reference's gradients bit for bit).
struct HostGradGeom {
    std::vector<int32_t> nb;       // per entry: neighbour cell or -1-face
    std::vector<double> lsq_w;     // per entry [2]: w*dx, w*dy (w = 1/d^2)
    std::vector<double> lsq_inv;   // per cell [3]: inv00, inv01, inv11
    std::vector<double> gg;        // per entry [4]: outward nx, ny, length, owner weight w_c
    std::vector<double> fgrad;     // per face [8]: dist, cos_theta, kx, ky, w_L, nd, nx, ny
};
void build_grad_geom(const HostMesh& m, HostGradGeom& g);

// Concatenation of independent meshes (batched solves): nodes, faces and
// cells of mesh k follow those of mesh k-1 with offset indices; patch ids
// are shared (every part must have the same patch count).
void concat_meshes(const std::vector<const HostMesh*>& parts, HostMesh& out);

// Agglomeration multigrid: the next coarser level of `fine`.  agg[c] is
// the agglomerate of fine cell c (reference numbering of both).  Each
// coarse face merges the fine faces between two agglomerates (or one
// agglomerate and one patch): area-weighted normal and midpoint, length
// |sum n_f A_f|; coarse cells carry the summed volume and the
// volume-weighted centroid.  The result has no nodes and needs
// build_device_layout before use.
void agglomerate(const HostMesh& fine, std::vector<int32_t>& agg, HostMesh& coarse);

// src/MeshReader.cpp:317-456 (+ validate_mesh_geometry :125-288).
// Throws MeshError on invalid input.
void build_from_polygons(HostMesh& m, int32_t n_nodes, const double* xy, int32_t n_cells, const int64_t* cell_off,
                         const int32_t* cell_nodes, int32_t n_bedges, const int32_t* bedge_nodes,
                         const int32_t* bedge_patch, int32_t n_patches);

void build_from_faces(HostMesh& m, int32_t n_nodes, const double* xy, int32_t n_faces, const int32_t* face_nodes,
                      const int32_t* face_cells, const int32_t* face_patch, int32_t n_cells,
                      const int32_t* cell_face_off, const int32_t* cell_faces, const double* cell_geom,
                      int32_t n_patches);

}  // namespace fvgb
