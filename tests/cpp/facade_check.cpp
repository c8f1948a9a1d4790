// Checks of the C++ facade (include/aep/hybrid_solver.hpp), driven by
// tests/test_facade.py.
//
//   facade_check host <dir>   host logic only (no device calls): ObjMesh parsing and
//                             mesh rules, RegularGrid indexing, scene factories,
//                             frame-file format
//   facade_check gpu <dir>    a SandCylinder scene through HybridSolver: dumps the
//                             initial and stepped state for the Python side to
//                             replay through ctypes, checkpoint resume, solve()
//                             with frame files, the weight query
//
// Prints "OK <mode>" and key=value lines; exits nonzero on the first failure.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "aep/hybrid_solver.hpp"

namespace {

int failures = 0;
#define EXPECT(c)                                                               \
    do {                                                                        \
        if (!(c)) {                                                             \
            std::cerr << "FAIL " << __FILE__ << ":" << __LINE__ << ": " #c "\n"; \
            ++failures;                                                         \
        }                                                                       \
    } while (0)

bool near(double a, double b, double tol) { return std::fabs(a - b) <= tol * std::max(1.0, std::fabs(b)); }

void write_raw(std::ofstream& out, const double* p, size_t n) {
    out.write(reinterpret_cast<const char*>(p), (std::streamsize)(sizeof(double) * n));
}

int count_lines(const std::string& path, char first) {
    std::ifstream in(path);
    std::string line;
    int c = 0;
    while (std::getline(in, line))
        if (!line.empty() && line[0] == first) ++c;
    return c;
}

void host_checks(const std::string& dir) {
    // ObjMesh: unit right triangles of a 2x2 quad grid, with the records the
    // reference skips (comments, vn, vt) and "a/b/c" face tokens
    const std::string obj = dir + "/quad.obj";
    {
        std::ofstream o(obj);
        o << "# test mesh\nv 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1 0\nvn 0 0 1\nvt 0 0\n"
          << "f 1 2 3\nf 2/2/1 4/4/1 3/3/1\ng group\n";
    }
    aep::LagrangianMesh m = aep::LagrangianMesh::ObjMesh(obj, 2.0, 0.1, 200.0, 0.3, 5.0, 4e4, 45.0);
    EXPECT(m.vertexNumber() == 4 && m.elementNumber() == 2);
    EXPECT(m.faces(1, 0) == 1 && m.faces(1, 1) == 3 && m.faces(1, 2) == 2);
    EXPECT(near(m.elementVolumes[0], 0.25 * 0.5 * 0.1, 1e-12));
    EXPECT(near(m.vertexVolumes[1], 2 * 0.25 * 0.5 * 0.1, 1e-12));  // shared by both triangles
    EXPECT(near(m.vertexMasses[0], 2.0 * 0.25 * 0.5 * 0.1, 1e-12));
    EXPECT(near(m.elementRestDirections_3(0, 2), 1.0, 1e-12));     // unit normal +z
    EXPECT(near(m.elementRestDirections_1(1, 0), 0.0, 1e-12) && near(m.elementRestDirections_1(1, 1), 1.0, 1e-12));
    EXPECT(near(m.mu, 200.0 / 2.6, 1e-12) && near(m.lambda, 200.0 * 0.3 / 1.3 / 0.4, 1e-12));
    EXPECT(near(m.frictionCoeff, 1.0, 1e-12));
    EXPECT(near(m.elementPositions(0, 0), 1.0 / 3.0, 1e-12));
    bool threw = false;
    try {
        aep::LagrangianMesh::ObjMesh(dir + "/missing.obj", 1, 1, 1, 0.3, 1, 1, 0);
    } catch (const aep::Error& e) {
        threw = e.status == AEP_INVALID_ARG;
    }
    EXPECT(threw);
    std::vector<double> fixed(3, 1.0);
    threw = false;
    try {
        m.bindConstraints(&fixed);
    } catch (const aep::Error&) {
        threw = true;
    }
    EXPECT(threw);
    fixed.assign(4, 0.0);
    fixed[2] = 1.0;
    m.bindConstraints(&fixed);
    EXPECT(m.vertexIsFixed(2) && !m.vertexIsFixed(0));

    // RegularGrid
    aep::RegularGrid rg({0, 0, 0}, {1, 2, 3}, {4, 5, 6});
    EXPECT(rg.gridNumber() == 120);
    int i, j, k;
    std::tie(i, j, k) = rg.toCoordinate(rg.toIndex(3, 2, 5));
    EXPECT(i == 3 && j == 2 && k == 5);
    EXPECT(near(rg.h()[1], 0.4, 1e-15) && near(rg.positions()(rg.toIndex(1, 1, 1), 2), 0.5, 1e-15));

    // factories: counts, support, total mass, the hole of SandBlock
    aep::ParticleSystem sb = aep::ParticleSystem::SnowBall({0.5, 0.5, 0.5}, 0.1, 5000, 1);
    double mass = 0;
    for (double x : sb.masses) mass += x;
    EXPECT(sb.size() == 5000 && near(mass, 100.0 * 3.14 * 1e-3, 1e-12) && sb.material[0] == AEP_SNOW);
    double rmax = 0;
    for (size_t p = 0; p < sb.size(); ++p) {
        aep::Vec3 d{sb.positions(p, 0) - 0.5, sb.positions(p, 1) - 0.5, sb.positions(p, 2) - 0.5};
        rmax = std::max(rmax, std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]));
    }
    EXPECT(rmax <= 0.1 && rmax > 0.09);
    aep::ParticleSystem blk = aep::ParticleSystem::SandBlock({0, 0, 0}, {0.4, 0.4, 0.4}, 0.15, 8000, 2);
    bool hole_empty = true;
    for (size_t p = 0; p < blk.size(); ++p) {
        double dx = blk.positions(p, 0), dy = blk.positions(p, 1), dz = blk.positions(p, 2) - 0.2;
        if (dx * dx + dy * dy + dz * dz < 0.15 * 0.15) hole_empty = false;
    }
    EXPECT(hole_empty && blk.material[0] == AEP_SAND);
    aep::ParticleSystem cyl = aep::ParticleSystem::SandCylinder({0.5, 0.5, 0.1}, 0.1, 0.3, 3000, 3);
    EXPECT(cyl.velocities(7, 2) == -1.0 && cyl.positions(7, 2) >= 0.1 && cyl.positions(7, 2) < 0.4);
    aep::ParticleSystem cyl2 = aep::ParticleSystem::SandCylinder({0.5, 0.5, 0.1}, 0.1, 0.3, 3000, 3);
    EXPECT(cyl2.positions(2999, 0) == cyl.positions(2999, 0));  // seeded: reproducible
    threw = false;
    try {
        aep::ParticleSystem::SandBlock({0, 0, 0}, {1, 1, 0.2}, 0.1, 10, 0);
    } catch (const aep::Error&) {
        threw = true;
    }
    EXPECT(threw);

    // frame files
    aep::writeMeshObj(dir + "/frame.obj", m);
    EXPECT(count_lines(dir + "/frame.obj", 'v') == 4 && count_lines(dir + "/frame.obj", 'f') == 2);
    aep::LagrangianMesh back = aep::LagrangianMesh::ObjMesh(dir + "/frame.obj", 2.0, 0.1, 200.0, 0.3, 5.0, 4e4, 45.0);
    EXPECT(back.faces(1, 1) == 3 && back.vertexPositions(3, 1) == 1.0);
}

void dump_state(const std::string& path, const aep::ParticleSystem& ps) {
    std::ofstream out(path, std::ios::binary);
    const size_t n = ps.size();
    write_raw(out, ps.positions.data(), 3 * n);
    write_raw(out, ps.velocities.data(), 3 * n);
    write_raw(out, ps.affineMomenta_1.data(), 3 * n);
    write_raw(out, ps.affineMomenta_2.data(), 3 * n);
    write_raw(out, ps.affineMomenta_3.data(), 3 * n);
    for (size_t p = 0; p < n; ++p) write_raw(out, ps.elasticDeformationGradients[p].data(), 9);
    write_raw(out, ps.masses.data(), n);
    write_raw(out, ps.volumes.data(), n);
    write_raw(out, ps.plasticAmount.data(), n);
}

bool same(const aep::ParticleSystem& a, const aep::ParticleSystem& b) {
    const size_t n = a.size();
    if (std::memcmp(a.positions.data(), b.positions.data(), sizeof(double) * 3 * n) != 0) return false;
    if (std::memcmp(a.velocities.data(), b.velocities.data(), sizeof(double) * 3 * n) != 0) return false;
    for (size_t p = 0; p < n; ++p)
        if (a.elasticDeformationGradients[p] != b.elasticDeformationGradients[p]) return false;
    return std::memcmp(a.plasticAmount.data(), b.plasticAmount.data(), sizeof(double) * n) == 0;
}

void gpu_checks(const std::string& dir) {
    const int n = 20000;
    const double dt = 1e-4;
    aep::RegularGrid rg({0, 0, 0}, {1, 1, 1}, {32, 32, 32});
    aep::ParticleSystem ps = aep::ParticleSystem::SandCylinder({0.5, 0.5, 0.1}, 0.1, 0.25, n, 11);
    dump_state(dir + "/init.bin", ps);
    aep::HybridSolver solver(&ps, &rg);
    solver.setLevelSet(aep::LevelSet::ground(0.05) | aep::LevelSet::sphere({0.5, 0.5, 0.02}, 0.05));
    solver.initVolumes();
    for (int s = 0; s < 20; ++s) solver.step(dt);
    solver.pull();
    dump_state(dir + "/stepped.bin", ps);
    std::printf("steps=20 mass=%.17g\n", solver.stats().total_mass);

    // checkpoint: 10 more steps after a save equal 10 steps after a load
    solver.saveCheckpoint(dir + "/state.aep");
    for (int s = 0; s < 10; ++s) solver.step(dt);
    solver.pull();
    aep::ParticleSystem after = ps;
    aep::ParticleSystem ps2 = ps;
    aep::HybridSolver resumed(&ps2, &rg);
    resumed.loadCheckpoint(dir + "/state.aep");
    for (int s = 0; s < 10; ++s) resumed.step(dt);
    resumed.pull();
    EXPECT(same(after, ps2));

    // weight query: partition of unity for a particle away from the walls
    aep::HybridSolver::WeightRow row = solver.weights(5);
    double sw = 0;
    int nodes = 0;
    for (int k = 0; k < 64; ++k) {
        sw += row.w[k];
        nodes += row.node[k] >= 0;
    }
    EXPECT(std::fabs(sw - 1.0) < 1e-5 && nodes >= 27);

    // solve with frame files: maxt = 0.02 runs two 1/60 s frames
    aep::ParticleSystem ps3 = aep::ParticleSystem::SandCylinder({0.5, 0.5, 0.1}, 0.1, 0.25, n, 11);
    aep::HybridSolver sv(&ps3, &rg);
    sv.setLevelSet(aep::LevelSet::ground(0.05));
    sv.setOutputDirectory(dir + "/frames");
    std::vector<double> frame_t;
    sv.setFrameCallback([&](int, double t) {
        frame_t.push_back(t);
        return true;
    });
    sv.solve(0.3, 0.02, 0.95);
    const aep_solve_state st = sv.solveState();
    EXPECT(st.frames == 2 && frame_t.size() == 2);
    EXPECT(std::fabs(st.t - 2.0 / 60.0) < 1e-12);
    EXPECT(count_lines(dir + "/frames/particle/particle_0.obj", 'v') == n);
    EXPECT(count_lines(dir + "/frames/particle/particle_1.obj", 'v') == n);
    std::printf("solve_steps=%lld frames=%d t=%.17g dt=%.17g\n", (long long)st.steps, st.frames, st.t, st.dt);
    double zmin = 1e9;
    for (int p = 0; p < n; ++p) zmin = std::min(zmin, ps3.positions(p, 2));
    EXPECT(zmin > 0.03);  // resting on the ground
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: facade_check host|gpu <dir>\n");
        return 2;
    }
    const std::string mode = argv[1], dir = argv[2];
    try {
        if (mode == "host")
            host_checks(dir);
        else if (mode == "gpu")
            gpu_checks(dir);
        else
            return 2;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "exception: %s\n", e.what());
        return 1;
    }
    if (failures) return 1;
    std::printf("OK %s\n", mode.c_str());
    return 0;
}
