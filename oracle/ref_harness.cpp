// Driver for the reference solver classes, compiled in place from the
// reference's own sources (see oracle/Makefile).  This file is test
// infrastructure: it runs the reference's EulerFVMSolver /
// NavierStokesFVMSolver / UnstructuredFVMSolver / GradientCalculator /
// compute_wall_distance on a .fvmesh and dumps raw little-endian binaries
// that the parity tests and the golden-fixture script read.
//
// Usage: fvref <mode> mesh=<file.fvmesh> out=<dir> [key=value ...]
//   mode = mesh | euler | ns | rans | diff | grad | walldist
// Reference interfaces driven here:
//   MeshReader::read               include/MeshReader.h:81
//   EulerFVMSolver                 include/EulerFVMSolver.h:107-160
//   NavierStokesFVMSolver          include/NavierStokesFVMSolver.h:118-218
//   UnstructuredFVMSolver          include/UnstructuredFVMSolver.h:34-73
//   GradientCalculator, face_gradient, corrected_face_gradient_vector,
//   face_normal_distance           include/GradientReconstruction.h:46-162
//   compute_wall_forces            include/WallTraction.h:143
//   compute_wall_distance          include/WallDistance.h:38
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "CflRamp.h"
#include "Checkpoint.h"
#include "EulerFVMSolver.h"
#include "GradientReconstruction.h"
#include "MeshReader.h"
#include "NavierStokesFVMSolver.h"
#include "UnstructuredFVMSolver.h"
#include "RANSTurbulenceSASolver.h"
#include "WallDistance.h"
#include "WallTraction.h"

namespace {

std::map<std::string, std::vector<std::string>> g_args;

std::string arg(const std::string& k, const std::string& dflt = "") {
    auto it = g_args.find(k);
    if (it == g_args.end() || it->second.empty()) return dflt;
    return it->second.back();
}
double argd(const std::string& k, double dflt) {
    std::string s = arg(k);
    return s.empty() ? dflt : std::strtod(s.c_str(), nullptr);
}
long argi(const std::string& k, long dflt) {
    std::string s = arg(k);
    return s.empty() ? dflt : std::strtol(s.c_str(), nullptr, 10);
}
std::vector<std::string> split(const std::string& s, char sep) {
    std::vector<std::string> out;
    std::stringstream ss(s);
    std::string item;
    while (std::getline(ss, item, sep)) out.push_back(item);
    return out;
}

template <typename T>
void dump(const std::string& path, const std::vector<T>& v) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) { std::perror(path.c_str()); std::exit(3); }
    if (!v.empty()) std::fwrite(v.data(), sizeof(T), v.size(), f);
    std::fclose(f);
}

int patch_index(const UnstructuredMesh& m, const std::string& name) {
    for (size_t i = 0; i < m.patches.size(); ++i)
        if (m.patches[i].name == name) return (int)i;
    return -1;
}

NumericalFluxScheme flux_of(const std::string& s) {
    if (s == "hllc") return NumericalFluxScheme::HLLC;
    if (s == "exact") return NumericalFluxScheme::Exact;
    return NumericalFluxScheme::Rusanov;
}

EulerInitialCondition ic_from_args() {
    EulerInitialCondition ic;
    std::vector<std::string> p = split(arg("ic", "free:1:0:0:1"), ':');
    if (p[0] == "two") {
        ic.mode = EulerICMode::TwoRegion;
        ic.rho_l = std::stod(p[1]); ic.u_l = std::stod(p[2]); ic.v_l = std::stod(p[3]); ic.p_l = std::stod(p[4]);
        ic.rho_r = std::stod(p[5]); ic.u_r = std::stod(p[6]); ic.v_r = std::stod(p[7]); ic.p_r = std::stod(p[8]);
        ic.x0 = std::stod(p[9]);
    } else {
        ic.mode = EulerICMode::Freestream;
        ic.rho = std::stod(p[1]); ic.u = std::stod(p[2]); ic.v = std::stod(p[3]); ic.p = std::stod(p[4]);
    }
    return ic;
}

void dump_history(const std::string& out, const std::vector<double>& hist, double secs, long steps, size_t n) {
    dump(out + "/resid.f64", hist);
    std::printf("{\"steps\": %ld, \"cells\": %zu, \"seconds\": %.6f}\n", steps, n, secs);
}

int run_mesh(const UnstructuredMesh& m, const std::string& out) {
    std::vector<int> fi;
    std::vector<double> fd;
    for (const Face& f : m.faces) {
        fi.insert(fi.end(), {f.node1, f.node2, f.cell_left, f.cell_right, f.patch_id});
        fd.insert(fd.end(), {f.nx, f.ny, f.area, f.x_mid, f.y_mid});
    }
    std::vector<double> cd;
    std::vector<int> off{0}, cf;
    for (const Cell& c : m.cells) {
        cd.insert(cd.end(), {c.volume, c.x_centroid, c.y_centroid});
        cf.insert(cf.end(), c.faces.begin(), c.faces.end());
        off.push_back((int)cf.size());
    }
    dump(out + "/faces_i32.bin", fi);
    dump(out + "/faces_f64.bin", fd);
    dump(out + "/cells_f64.bin", cd);
    dump(out + "/cell_face_off.bin", off);
    dump(out + "/cell_faces.bin", cf);
    std::ofstream pn(out + "/patches.txt");
    for (const BoundaryPatch& p : m.patches) pn << p.name << "\n";
    std::printf("{\"cells\": %zu, \"faces\": %zu, \"patches\": %zu}\n", m.cells.size(), m.faces.size(),
                m.patches.size());
    return 0;
}

int run_euler(const UnstructuredMesh& m, const std::string& out) {
    double gamma = argd("gamma", 1.4);
    std::vector<EulerBoundaryCondition> bcs(m.patches.size());
    for (const std::string& spec : g_args["bc"]) {
        std::vector<std::string> p = split(spec, ':');
        int pid = patch_index(m, p[0]);
        if (pid < 0) { std::fprintf(stderr, "unknown patch %s\n", p[0].c_str()); return 2; }
        if (p[1] == "wall") bcs[pid].type = EulerBoundaryType::Wall;
        else if (p[1] == "outflow") bcs[pid].type = EulerBoundaryType::Outflow;
        else {
            bcs[pid].type = EulerBoundaryType::Farfield;
            bcs[pid].farfield_state = from_primitive(std::stod(p[2]), std::stod(p[3]), std::stod(p[4]),
                                                     std::stod(p[5]), gamma);
        }
    }
    EulerFVMSolver solver(m, bcs, gamma, argd("cfl", 0.5), ic_from_args(), flux_of(arg("flux", "rusanov")),
                          argd("tol", 1e-6), (int)argi("maxit", 20));
    long steps = argi("steps", 10);
    std::vector<double> hist;
    hist.reserve(steps * 4);
    auto t0 = std::chrono::steady_clock::now();
    for (long s = 0; s < steps; ++s) {
        solver.step();
        const EulerResidualNorms& r = solver.residual();
        hist.insert(hist.end(), {r.rho, r.rho_u, r.rho_v, r.E});
    }
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::vector<double> field;
    for (const EulerState& s : solver.field()) field.insert(field.end(), {s.rho, s.rho_u, s.rho_v, s.E});
    dump(out + "/field.f64", field);
    if (!arg("ref_rho").empty()) {
        // Inviscid wall forces: compute_wall_traction over every slip-wall
        // face with zero viscosity and zero gradients (the traction is then
        // the owner cell's pressure alone), then compute_wall_forces.
        const size_t N = m.cells.size();
        std::vector<double> u(N), v(N), p(N), rho(N), mu0(N, 0.0);
        std::vector<Gradient2> g0(N);
        for (size_t c = 0; c < N; ++c) {
            const EulerState& s = solver.field()[c];
            rho[c] = s.rho;
            u[c] = s.rho_u / s.rho;
            v[c] = s.rho_v / s.rho;
            p[c] = pressure(s, gamma);
        }
        std::vector<int> wall_faces;
        for (size_t f = 0; f < m.faces.size(); ++f)
            if (m.faces[f].cell_right == -1 && bcs[m.faces[f].patch_id].type == EulerBoundaryType::Wall)
                wall_faces.push_back((int)f);
        UnstructuredMesh mg = m;
        mg.compute_geometry();
        std::vector<double> bz(m.faces.size(), 0.0);
        std::vector<WallFaceSample> samples =
            compute_wall_traction(mg, wall_faces, u, v, p, rho, mu0, bz, bz, g0, g0);
        WallReferenceQuantities ref;
        ref.rho_ref = argd("ref_rho", 1.0);
        ref.velocity_x_ref = argd("ref_u", 1.0);
        ref.velocity_y_ref = argd("ref_v", 0.0);
        ref.p_ref = argd("ref_p", 0.0);
        ref.length_ref = argd("ref_len", 1.0);
        ref.moment_reference_x = argd("ref_mx", 0.25);
        ref.moment_reference_y = argd("ref_my", 0.0);
        std::vector<double> forces;
        for (const WallForceReport& r : compute_wall_forces(mg, samples, ref))
            forces.insert(forces.end(), {(double)r.patch_id, r.friction_drag, r.pressure_drag, r.total_drag, r.lift,
                                         r.moment, r.cd_friction, r.cd_pressure, r.cd_total, r.cl, r.cm});
        dump(out + "/forces.f64", forces);
    }
    dump_history(out, hist, secs, steps, m.cells.size());
    return 0;
}

int run_ns(const UnstructuredMesh& m, const std::string& out) {
    double gamma = argd("gamma", 1.4);
    std::vector<NSBoundaryCondition> bcs(m.patches.size());
    std::vector<int> wall_faces;
    for (const std::string& spec : g_args["bc"]) {
        std::vector<std::string> p = split(spec, ':');
        int pid = patch_index(m, p[0]);
        if (pid < 0) { std::fprintf(stderr, "unknown patch %s\n", p[0].c_str()); return 2; }
        NSBoundaryCondition& bc = bcs[pid];
        if (p[1] == "noslip") {
            bc.type = NSBoundaryType::NoSlipWall;
            if (p.size() > 2) bc.wall_u = std::stod(p[2]);
            if (p.size() > 3) bc.wall_v = std::stod(p[3]);
            if (p.size() > 4) { bc.is_isothermal_wall = true; bc.wall_temperature = std::stod(p[4]); }
        } else if (p[1] == "outflow") {
            bc.type = NSBoundaryType::Outflow;
        } else {
            bc.type = NSBoundaryType::Farfield;
            bc.farfield_state = from_primitive(std::stod(p[2]), std::stod(p[3]), std::stod(p[4]),
                                               std::stod(p[5]), gamma);
        }
    }
    for (size_t f = 0; f < m.faces.size(); ++f) {
        const Face& face = m.faces[f];
        if (face.cell_right == -1 && bcs[face.patch_id].type == NSBoundaryType::NoSlipWall)
            wall_faces.push_back((int)f);
    }
    GradientScheme gs = arg("grad", "lsq") == "gg" ? GradientScheme::GreenGauss : GradientScheme::LeastSquares;
    NavierStokesFVMSolver solver(m, bcs, gamma, argd("R", 287.0), argd("mu", 1e-3), argd("Pr", 0.72),
                                 argd("cfl", 0.5), ic_from_args(), flux_of(arg("flux", "rusanov")), gs,
                                 argd("tol", 1e-6), (int)argi("maxit", 20));
    long steps = argi("steps", 10);
    std::vector<double> hist;
    auto t0 = std::chrono::steady_clock::now();
    for (long s = 0; s < steps; ++s) {
        solver.step();
        const EulerResidualNorms& r = solver.residual();
        hist.insert(hist.end(), {r.rho, r.rho_u, r.rho_v, r.E});
    }
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::vector<double> field;
    for (const EulerState& s : solver.field()) field.insert(field.end(), {s.rho, s.rho_u, s.rho_v, s.E});
    dump(out + "/field.f64", field);
    // Wall forces over every no-slip face: one report per patch + the total.
    std::vector<WallFaceSample> samples = solver.compute_wall_traction_samples(wall_faces);
    UnstructuredMesh mg = m;
    mg.compute_geometry();
    WallReferenceQuantities ref;
    ref.rho_ref = argd("ref_rho", 1.0);
    ref.velocity_x_ref = argd("ref_u", 1.0);
    ref.velocity_y_ref = argd("ref_v", 0.0);
    ref.p_ref = argd("ref_p", 0.0);
    ref.length_ref = argd("ref_len", 1.0);
    ref.moment_reference_x = argd("ref_mx", 0.25);
    ref.moment_reference_y = argd("ref_my", 0.0);
    std::vector<double> forces;
    for (const WallForceReport& r : compute_wall_forces(mg, samples, ref))
        forces.insert(forces.end(), {(double)r.patch_id, r.friction_drag, r.pressure_drag, r.total_drag, r.lift,
                                     r.moment, r.cd_friction, r.cd_pressure, r.cd_total, r.cl, r.cm});
    dump(out + "/forces.f64", forces);
    std::vector<double> tau;
    for (const WallFaceSample& s : samples) tau.insert(tau.end(), {(double)s.face_index, s.p, s.tau_wall});
    dump(out + "/wall.f64", tau);
    dump_history(out, hist, secs, steps, m.cells.size());
    return 0;
}

// RANSTurbulenceSASolver (include/RANSTurbulenceSASolver.h:1-233): bc specs
// as run_ns, farfield specs carry the freestream nut as a 7th field.
int run_rans(const UnstructuredMesh& m, const std::string& out) {
    double gamma = argd("gamma", 1.4);
    std::vector<RANSBoundaryConditionSA> bcs(m.patches.size());
    std::vector<int> wall_faces;
    for (const std::string& spec : g_args["bc"]) {
        std::vector<std::string> p = split(spec, ':');
        int pid = patch_index(m, p[0]);
        if (pid < 0) { std::fprintf(stderr, "unknown patch %s\n", p[0].c_str()); return 2; }
        NSBoundaryCondition& bc = bcs[pid].ns;
        if (p[1] == "noslip") {
            bc.type = NSBoundaryType::NoSlipWall;
            if (p.size() > 2) bc.wall_u = std::stod(p[2]);
            if (p.size() > 3) bc.wall_v = std::stod(p[3]);
            if (p.size() > 4) { bc.is_isothermal_wall = true; bc.wall_temperature = std::stod(p[4]); }
        } else if (p[1] == "outflow") {
            bc.type = NSBoundaryType::Outflow;
        } else {
            bc.type = NSBoundaryType::Farfield;
            bc.farfield_state = from_primitive(std::stod(p[2]), std::stod(p[3]), std::stod(p[4]),
                                               std::stod(p[5]), gamma);
            if (p.size() > 6) bcs[pid].farfield_nut = std::stod(p[6]);
        }
    }
    for (size_t f = 0; f < m.faces.size(); ++f) {
        const Face& face = m.faces[f];
        if (face.cell_right == -1 && bcs[face.patch_id].ns.type == NSBoundaryType::NoSlipWall)
            wall_faces.push_back((int)f);
    }
    GradientScheme gs = arg("grad", "lsq") == "gg" ? GradientScheme::GreenGauss : GradientScheme::LeastSquares;
    RANSTurbulenceSASolver solver(m, bcs, gamma, argd("R", 287.0), argd("mu", 1e-3), argd("Pr", 0.72),
                                  argd("Prt", 0.9), argd("cfl", 0.5), ic_from_args(), argd("nut0", 0.0),
                                  flux_of(arg("flux", "rusanov")), gs, argd("tol", 1e-6), (int)argi("maxit", 20));
    long steps = argi("steps", 10);
    std::vector<double> hist;
    auto t0 = std::chrono::steady_clock::now();
    for (long s = 0; s < steps; ++s) {
        solver.step();
        const EulerResidualNorms& r = solver.residual();
        hist.insert(hist.end(), {r.rho, r.rho_u, r.rho_v, r.E, solver.nut_residual()});
    }
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::vector<double> field;
    for (const EulerState& s : solver.field()) field.insert(field.end(), {s.rho, s.rho_u, s.rho_v, s.E});
    dump(out + "/field.f64", field);
    dump(out + "/nut.f64", solver.nut_field());
    std::vector<WallFaceSample> samples = solver.compute_wall_traction_samples(wall_faces);
    UnstructuredMesh mg = m;
    mg.compute_geometry();
    WallReferenceQuantities ref;
    ref.rho_ref = argd("ref_rho", 1.0);
    ref.velocity_x_ref = argd("ref_u", 1.0);
    ref.velocity_y_ref = argd("ref_v", 0.0);
    ref.p_ref = argd("ref_p", 0.0);
    ref.length_ref = argd("ref_len", 1.0);
    ref.moment_reference_x = argd("ref_mx", 0.25);
    ref.moment_reference_y = argd("ref_my", 0.0);
    std::vector<double> forces;
    for (const WallForceReport& r : compute_wall_forces(mg, samples, ref))
        forces.insert(forces.end(), {(double)r.patch_id, r.friction_drag, r.pressure_drag, r.total_drag, r.lift,
                                     r.moment, r.cd_friction, r.cd_pressure, r.cd_total, r.cl, r.cm});
    dump(out + "/forces.f64", forces);
    dump(out + "/walld.f64", compute_wall_distance(mg, wall_faces));
    std::vector<double> hist5(hist);
    {
        FILE* f = std::fopen((out + "/history.f64").c_str(), "wb");
        if (f) { std::fwrite(hist5.data(), sizeof(double), hist5.size(), f); std::fclose(f); }
    }
    std::printf("{\"steps\": %ld, \"cells\": %zu, \"seconds\": %.6f}\n", steps, m.cells.size(), secs);
    return 0;
}

// next_cfl (src/CflRamp.cpp:7-27) on the sequences of a binary file:
// per record [cfl, cfl_max, cfl_min, growth, shrink, divergence, window, n,
// history[n]] -> one output double each.
int run_cflramp() {
    std::ifstream in(arg("in"), std::ios::binary);
    std::vector<double> out;
    double head[8];
    while (in.read(reinterpret_cast<char*>(head), sizeof(head))) {
        std::vector<double> h((size_t)head[7]);
        in.read(reinterpret_cast<char*>(h.data()), sizeof(double) * h.size());
        CflRampParams p;
        p.cfl_min = head[2];
        p.growth_factor = head[3];
        p.shrink_factor = head[4];
        p.divergence_threshold = head[5];
        p.window = (int)head[6];
        out.push_back(next_cfl(head[0], head[1], h, p));
    }
    dump(arg("out"), out);
    std::printf("{\"records\": %zu}\n", out.size());
    return 0;
}

int run_diff(UnstructuredMesh m, const std::string& out) {
    for (const std::string& spec : g_args["bc"]) {
        std::vector<std::string> p = split(spec, ':');
        int pid = patch_index(m, p[0]);
        if (pid < 0) { std::fprintf(stderr, "unknown patch %s\n", p[0].c_str()); return 2; }
        m.patches[pid].type = (p[1] == "neumann") ? BoundaryType::Neumann : BoundaryType::Dirichlet;
        m.patches[pid].value = std::stod(p[2]);
    }
    UnstructuredFVMSolver solver(m, argd("alpha", 1.0), argd("dt", 1e-4), argd("v0", 1.0), argd("r0", 0.5));
    long steps = argi("steps", 10);
    std::vector<double> hist;
    auto t0 = std::chrono::steady_clock::now();
    for (long s = 0; s < steps; ++s) {
        solver.step();
        hist.push_back(solver.residual_norm());
    }
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    dump(out + "/field.f64", solver.field());
    dump_history(out, hist, secs, steps, m.cells.size());
    return 0;
}

// phi(x, y) = c0 + c1 x + c2 y + c3 x^2 + c4 x y + c5 y^2
double poly(const std::vector<double>& c, double x, double y) {
    return c[0] + c[1] * x + c[2] * y + c[3] * x * x + c[4] * x * y + c[5] * y * y;
}

int run_grad(UnstructuredMesh m, const std::string& out) {
    m.compute_geometry();
    std::vector<double> c(6, 0.0);
    std::vector<std::string> p = split(arg("phi", "1:2:3:0:0:0"), ':');
    for (size_t i = 0; i < p.size() && i < 6; ++i) c[i] = std::stod(p[i]);
    std::vector<double> phi(m.cells.size()), bphi(m.faces.size(), 0.0);
    for (size_t i = 0; i < m.cells.size(); ++i) phi[i] = poly(c, m.cells[i].x_centroid, m.cells[i].y_centroid);
    for (size_t f = 0; f < m.faces.size(); ++f)
        if (m.faces[f].cell_right == -1) bphi[f] = poly(c, m.faces[f].x_mid, m.faces[f].y_mid);
    GradientScheme gs = arg("grad", "lsq") == "gg" ? GradientScheme::GreenGauss : GradientScheme::LeastSquares;
    GradientCalculator calc(m, gs);
    std::vector<Gradient2> g = calc.compute(m, phi, bphi);
    std::vector<double> gd, fd;
    for (const Gradient2& q : g) gd.insert(gd.end(), {q.dphidx, q.dphidy});
    for (size_t f = 0; f < m.faces.size(); ++f) {
        const Face& face = m.faces[f];
        int cl = face.cell_left, cr = face.cell_right;
        bool b = cr == -1;
        FaceGradient fg = face_gradient(m, face, phi[cl], b ? 0.0 : phi[cr], g[cl], b ? Gradient2{} : g[cr], bphi[f]);
        Gradient2 cg = corrected_face_gradient_vector(fg, face.nx, face.ny);
        fd.insert(fd.end(), {fg.dphidn, cg.dphidx, cg.dphidy, face_normal_distance(m, face)});
    }
    dump(out + "/phi.f64", phi);
    dump(out + "/grad.f64", gd);
    dump(out + "/facegrad.f64", fd);
    std::printf("{\"cells\": %zu}\n", m.cells.size());
    return 0;
}

int run_walldist(UnstructuredMesh m, const std::string& out) {
    m.compute_geometry();
    std::vector<int> wall;
    for (const std::string& name : g_args["wall"]) {
        int pid = patch_index(m, name);
        for (size_t f = 0; f < m.faces.size(); ++f)
            if (m.faces[f].cell_right == -1 && m.faces[f].patch_id == pid) wall.push_back((int)f);
    }
    dump(out + "/walldist.f64", compute_wall_distance(m, wall));
    return 0;
}

// Checkpoint::write / Checkpoint::read (include/Checkpoint.h:72-116):
//   ckpt op=write path=<f> eq=<tag> step=<n> build=<b> in=<raw doubles> cells=<n>
//   ckpt op=read  path=<f> eq=<tag> cells=<n> out=<dir>   (prints step/build)
int run_ckpt() {
    const std::string path = arg("path");
    const CheckpointEquation eq = (CheckpointEquation)argi("eq", 1);
    const size_t cells = (size_t)argi("cells", 0);
    const bool flow = eq != CheckpointEquation::Diffusion && eq != CheckpointEquation::AdvectionDiffusion;
    if (arg("op") == "write") {
        std::ifstream in(arg("in"), std::ios::binary);
        std::vector<double> raw(cells * (flow ? 4 : 1));
        in.read(reinterpret_cast<char*>(raw.data()), (std::streamsize)(raw.size() * sizeof(double)));
        bool ok;
        if (flow) {
            std::vector<EulerState> U(cells);
            for (size_t i = 0; i < cells; ++i) U[i] = {raw[4 * i], raw[4 * i + 1], raw[4 * i + 2], raw[4 * i + 3]};
            ok = Checkpoint::write(path, eq, argi("step", 0), (unsigned long long)argi("build", 0), U);
        } else {
            ok = Checkpoint::write(path, eq, argi("step", 0), (unsigned long long)argi("build", 0), raw);
        }
        return ok ? 0 : 1;
    }
    long long step = 0;
    unsigned long long build = 0;
    std::vector<double> out;
    bool ok;
    if (flow) {
        std::vector<EulerState> U;
        ok = Checkpoint::read(path, eq, cells, step, build, U);
        for (const EulerState& s : U) out.insert(out.end(), {s.rho, s.rho_u, s.rho_v, s.E});
    } else {
        ok = Checkpoint::read(path, eq, cells, step, build, out);
    }
    if (!ok) return 1;
    dump(arg("out", ".") + "/payload.f64", out);
    std::printf("{\"step\": %lld, \"build\": %llu}\n", step, build);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: fvref <mesh|euler|ns|rans|diff|grad|walldist> mesh=<f> out=<dir> [k=v...]\n");
        return 2;
    }
    std::string mode = argv[1];
    for (int i = 2; i < argc; ++i) {
        const char* eq = std::strchr(argv[i], '=');
        if (!eq) continue;
        g_args[std::string(argv[i], eq - argv[i])].push_back(eq + 1);
    }
    if (mode == "ckpt") return run_ckpt();
    if (mode == "cflramp") return run_cflramp();
    UnstructuredMesh mesh;
    if (!MeshReader::read(arg("mesh"), mesh)) return 1;
    std::string out = arg("out", ".");
    if (mode == "mesh") { mesh.compute_geometry(); return run_mesh(mesh, out); }
    if (mode == "euler") return run_euler(mesh, out);
    if (mode == "ns") return run_ns(mesh, out);
    if (mode == "rans") return run_rans(mesh, out);
    if (mode == "diff") return run_diff(mesh, out);
    if (mode == "grad") return run_grad(mesh, out);
    if (mode == "walldist") return run_walldist(mesh, out);
    std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
    return 2;
}
