// Stand-in for the reference's include/UnstructuredMesh.h where the
// reference is not installed: the same struct shapes (include/
// UnstructuredMesh.h:20-63), declarations only, so the drop-in headers and
// a reference-style driver compile.
#ifndef UNSTRUCTUREDMESH_H_INCLUDED
#define UNSTRUCTUREDMESH_H_INCLUDED
#include <string>
#include <vector>
struct Node { double x, y; };
struct Face {
    int node1, node2;
    int cell_left;
    int cell_right;
    int patch_id = -1;
    double nx, ny;
    double area;
    double x_mid, y_mid;
};
struct Cell {
    double volume;
    double x_centroid;
    double y_centroid;
    std::vector<int> faces;
    std::vector<int> node_ids;
};
enum class BoundaryType : int { Dirichlet = 0, Neumann = 1 };
struct BoundaryPatch {
    std::string name;
    BoundaryType type = BoundaryType::Dirichlet;
    double value = 0.0;
};
struct UnstructuredMesh {
    std::vector<Node> nodes;
    std::vector<Face> faces;
    std::vector<Cell> cells;
    std::vector<BoundaryPatch> patches;
};
#endif
