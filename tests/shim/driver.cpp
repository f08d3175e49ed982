// A reference-style driver: written against the reference's class API
// (EulerFVMSolver / NavierStokesFVMSolver / UnstructuredFVMSolver with
// UnstructuredMesh), compiled against the GB300 drop-in headers.
//
//   driver <mesh.txt> <case.txt> <out.f64>
// mesh.txt: the mesh in reference numbering (nodes; faces node1 node2
// left right patch; cells volume cx cy nfaces faces...; patch names with
// diffusion type/value).  case.txt: "key value" lines.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <string>
#include <vector>

#include "EulerFVMSolver.h"
#include "NavierStokesFVMSolver.h"
#include "RANSTurbulenceSASolver.h"
#include "UnstructuredFVMSolver.h"

static UnstructuredMesh read_mesh(const char* path) {
    std::ifstream in(path);
    UnstructuredMesh m;
    size_t n;
    in >> n;
    m.nodes.resize(n);
    for (auto& p : m.nodes) in >> p.x >> p.y;
    in >> n;
    m.faces.resize(n);
    for (auto& f : m.faces) in >> f.node1 >> f.node2 >> f.cell_left >> f.cell_right >> f.patch_id;
    in >> n;
    m.cells.resize(n);
    for (auto& c : m.cells) {
        int k;
        in >> c.volume >> c.x_centroid >> c.y_centroid >> k;
        c.faces.resize(k);
        for (int& f : c.faces) in >> f;
    }
    in >> n;
    m.patches.resize(n);
    for (auto& p : m.patches) {
        int t;
        in >> p.name >> t >> p.value;
        p.type = t ? BoundaryType::Neumann : BoundaryType::Dirichlet;
    }
    return m;
}

int main(int argc, char** argv) {
    if (argc < 4) return 2;
    UnstructuredMesh mesh = read_mesh(argv[1]);
    std::map<std::string, double> kv;
    std::ifstream cf(argv[2]);
    std::string k;
    double v;
    while (cf >> k >> v) kv[k] = v;
    const double g = 1.4;
    const int steps = (int)kv["steps"];
    std::vector<double> out;
    EulerInitialCondition ic;
    ic.rho = kv["rho"]; ic.u = kv["u"]; ic.v = kv["v"]; ic.p = kv["p"];
    EulerState fs;
    fs.rho = ic.rho; fs.rho_u = ic.rho * ic.u; fs.rho_v = ic.rho * ic.v;
    fs.E = ic.p / (g - 1.0) + 0.5 * ic.rho * (ic.u * ic.u + ic.v * ic.v);
    const int kind = (int)kv["kind"];
    if (kind == 0) {
        std::vector<EulerBoundaryCondition> bcs(mesh.patches.size());
        bcs[0].type = EulerBoundaryType::Wall;
        bcs[1].type = EulerBoundaryType::Farfield;
        bcs[1].farfield_state = fs;
        EulerFVMSolver s(mesh, bcs, g, kv["cfl"], ic, (NumericalFluxScheme)(int)kv["flux"], 1e-6, 20);
        for (int i = 0; i < steps; ++i) s.step();
        for (const EulerState& q : s.field()) out.insert(out.end(), {q.rho, q.rho_u, q.rho_v, q.E});
        const EulerResidualNorms& r = s.residual();
        out.insert(out.end(), {r.rho, r.rho_u, r.rho_v, r.E});
    } else if (kind == 1) {
        std::vector<NSBoundaryCondition> bcs(mesh.patches.size());
        bcs[0].type = NSBoundaryType::NoSlipWall;
        bcs[1].type = NSBoundaryType::Farfield;
        bcs[1].farfield_state = fs;
        NavierStokesFVMSolver s(mesh, bcs, g, kv["R"], kv["mu"], kv["Pr"], kv["cfl"], ic,
                                (NumericalFluxScheme)(int)kv["flux"], GradientScheme::LeastSquares, 1e-6, 20);
        s.run(steps);
        for (const EulerState& q : s.field()) out.insert(out.end(), {q.rho, q.rho_u, q.rho_v, q.E});
        const EulerResidualNorms& r = s.residual();
        out.insert(out.end(), {r.rho, r.rho_u, r.rho_v, r.E});
    } else if (kind == 3) {
        std::vector<RANSBoundaryConditionSA> bcs(mesh.patches.size());
        bcs[0].ns.type = NSBoundaryType::NoSlipWall;
        bcs[1].ns.type = NSBoundaryType::Farfield;
        bcs[1].ns.farfield_state = fs;
        bcs[1].farfield_nut = kv["nut_far"];
        RANSTurbulenceSASolver s(mesh, bcs, g, kv["R"], kv["mu"], kv["Pr"], kv["Prt"], kv["cfl"], ic, kv["nut0"],
                                 (NumericalFluxScheme)(int)kv["flux"], GradientScheme::LeastSquares, 1e-6, 20);
        s.run(steps);
        for (const EulerState& q : s.field()) out.insert(out.end(), {q.rho, q.rho_u, q.rho_v, q.E});
        const std::vector<double>& nut = s.nut_field();
        out.insert(out.end(), nut.begin(), nut.end());
        const EulerResidualNorms& r = s.residual();
        out.insert(out.end(), {r.rho, r.rho_u, r.rho_v, r.E, s.nut_residual()});
    } else {
        UnstructuredFVMSolver s(mesh, kv["alpha"], kv["dt"], kv["v0"], kv["r0"]);
        s.run(steps);
        out = s.field();
        out.push_back(s.residual_norm());
    }
    FILE* f = std::fopen(argv[3], "wb");
    std::fwrite(out.data(), sizeof(double), out.size(), f);
    std::fclose(f);
    return 0;
}
