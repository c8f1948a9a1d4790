// hybrid_solver.hpp -- C++ host facade over the C-ABI of aep.h, with the class
// surface of the reference (HybridSolver.h, ParticleSystem.h, RegularGrid.h,
// LagrangianMesh.h, LevelSet.h), so that a program written against the
// reference's classes switches by changing includes and linking libaep.so.
//
// Header-only C++17, no Eigen.  Eigen's storage is kept where the reference
// exposes it:
//   Block3<double>  = Eigen::MatrixX3d (N x 3, column-major: all x, all y, all z)
//   Block3<int32_t> = Eigen::MatrixX3i (faces, 0-based vertex indices)
//   Mat3            = Eigen::Matrix3d   (3x3, column-major: M(a,b) at [a + 3b])
// so the arrays go to the C-ABI without repacking.
//
// Differences from the reference, by design:
//  * the state lives on the GPU: HybridSolver uploads the bound ParticleSystem /
//    LagrangianMesh at the first step and copies results back into their
//    members on pull() (solve() pulls at every frame and at its end);
//  * errors throw aep::Error instead of printing and spinning (RegularGrid.cpp:134,
//    LagrangianMesh.cpp:213,360,474) or exiting (ParticleSystem.cpp:255);
//  * the material is a per-particle tag (the reference's solve hard-codes SAND,
//    HybridSolver.cpp:873,955,959); factories tag their particles;
//  * scene factories take a seed (the reference seeds from the clock or not at all);
//  * ObjMesh reads 32-bit face indices (the reference reads unsigned short).
#pragma once

#include <sys/stat.h>

#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <functional>
#include <iterator>
#include <random>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "../aep.h"

namespace aep {

class Error : public std::runtime_error {
public:
    Error(aep_status st, const std::string& what) : std::runtime_error(what), status(st) {}
    aep_status status;
};

using Vec3 = std::array<double, 3>;
using Mat3 = std::array<double, 9>;  // column-major

inline Mat3 identity3() { return Mat3{1, 0, 0, 0, 1, 0, 0, 0, 1}; }

// N x 3 column-major block (Eigen::MatrixX3d / MatrixX3i storage)
template <class T>
class Block3 {
public:
    Block3() = default;
    explicit Block3(size_t n) : d_(3 * n, T(0)) {}
    size_t rows() const { return d_.size() / 3; }
    void resize(size_t n) { d_.assign(3 * n, T(0)); }  // new contents are zero
    void setZero() { std::fill(d_.begin(), d_.end(), T(0)); }
    T& operator()(size_t i, int c) { return d_[c * rows() + i]; }
    const T& operator()(size_t i, int c) const { return d_[c * rows() + i]; }
    std::array<T, 3> row(size_t i) const { return {(*this)(i, 0), (*this)(i, 1), (*this)(i, 2)}; }
    void setRow(size_t i, const std::array<T, 3>& v) {
        for (int c = 0; c < 3; ++c) (*this)(i, c) = v[c];
    }
    T* data() { return d_.data(); }
    const T* data() const { return d_.data(); }

private:
    std::vector<T> d_;
};

inline void check(aep_status st, aep_solver* s, const char* where) {
    if (st != AEP_OK) {
        std::string msg = where;
        const char* e = s ? aep_last_error(s) : nullptr;
        if (e && *e) msg += std::string(": ") + e;
        throw Error(st, msg);
    }
}

namespace detail {
constexpr double kPi = 3.14159265358979323846;
inline Vec3 sub(const Vec3& a, const Vec3& b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2]}; }
inline double norm(const Vec3& a) { return std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }
inline Vec3 cross(const Vec3& a, const Vec3& b) {
    return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}
// triangleArea: Heron's formula on the edge lengths (geometry.cpp:13-23)
inline double triangle_area(const Vec3& v1, const Vec3& v2, const Vec3& v3) {
    const double a = norm(sub(v2, v1)), b = norm(sub(v3, v2)), c = norm(sub(v1, v3));
    const double p = 0.5 * (a + b + c);
    return std::sqrt(p * (p - a) * (p - b) * (p - c));
}
// triangleNormal: normalised (v2 - v1) x (v3 - v1) (geometry.cpp:25-28)
inline Vec3 triangle_normal(const Vec3& v1, const Vec3& v2, const Vec3& v3) {
    Vec3 n = cross(sub(v2, v1), sub(v3, v1));
    const double l = norm(n);
    return {n[0] / l, n[1] / l, n[2] / l};
}
inline void make_dirs(const std::string& d) { ::mkdir(d.c_str(), 0755); }
}  // namespace detail

// ------------------------------------------------------------------------------------
// RegularGrid (RegularGrid.h:13-60, RegularGrid.cpp:117-200)
class RegularGrid {
public:
    RegularGrid(const Vec3& minBound, const Vec3& maxBound, const std::array<int, 3>& resolution)
        : min_(minBound), max_(maxBound), res_(resolution) {
        for (int a = 0; a < 3; ++a) {
            if (!(max_[a] > min_[a]) || res_[a] < 1)
                throw Error(AEP_INVALID_ARG, "RegularGrid: maxBound must exceed minBound and resolution be >= 1");
            h_[a] = (max_[a] - min_[a]) / res_[a];
        }
        masses.assign(gridNumber(), 0.0);
        velocities.resize(gridNumber());
        forces.resize(gridNumber());
    }
    int gridNumber() const { return res_[0] * res_[1] * res_[2]; }
    int toIndex(int i, int j, int k) const { return k * res_[0] * res_[1] + j * res_[0] + i; }
    std::tuple<int, int, int> toCoordinate(int index) const {
        const int k = index / (res_[0] * res_[1]);
        const int j = (index % (res_[0] * res_[1])) / res_[0];
        return std::make_tuple(index % res_[0], j, k);
    }
    const Vec3& h() const { return h_; }
    const Vec3& minBound() const { return min_; }
    const Vec3& maxBound() const { return max_; }
    const std::array<int, 3>& resolution() const { return res_; }
    Block3<double> positions() const {
        Block3<double> p((size_t)gridNumber());
        for (int k = 0; k < res_[2]; ++k)
            for (int j = 0; j < res_[1]; ++j)
                for (int i = 0; i < res_[0]; ++i)
                    p.setRow((size_t)toIndex(i, j, k), {min_[0] + i * h_[0], min_[1] + j * h_[1], min_[2] + k * h_[2]});
        return p;
    }
    double max_velocity() const {
        double m = 0.0;
        for (size_t i = 0; i < velocities.rows(); ++i) m = std::max(m, detail::norm(velocities.row(i)));
        return m;
    }
    double CFL_condition() const { return max_velocity() / std::min(h_[0], std::min(h_[1], h_[2])); }
    aep_grid_desc desc() const {
        aep_grid_desc g{};
        for (int a = 0; a < 3; ++a) {
            g.min[a] = min_[a];
            g.max[a] = max_[a];
            g.res[a] = res_[a];
        }
        return g;
    }

    // filled by HybridSolver::pullGrid()
    std::vector<double> masses;
    Block3<double> velocities;
    Block3<double> forces;

private:
    Vec3 min_, max_, h_{};
    std::array<int, 3> res_;
};

// ------------------------------------------------------------------------------------
// ParticleSystem (ParticleSystem.h:13-78, ParticleSystem.cpp:81-401)
class ParticleSystem {
public:
    std::vector<double> masses, volumes, densities, plasticAmount;
    Block3<double> velocities, positions;
    Block3<double> affineMomenta_1, affineMomenta_2, affineMomenta_3;
    std::vector<Mat3> elasticDeformationGradients, plasticDeformationGradients;
    std::vector<uint8_t> material;  // AEP_SNOW / AEP_SAND per particle
    double youngsModulus = 0, poissonRatio = 0, criticalCompression = 0, criticalStretch = 0, friction = 0;

    ParticleSystem() = default;
    // ParticleSystem(velocities, positions, Fe, Fp, masses, volumes, densities,
    // plasticAmount, E, nu, criticalCompression, criticalStretch, friction) (:81-117)
    ParticleSystem(const Block3<double>& v, const Block3<double>& x, const std::vector<Mat3>& Fe,
                   const std::vector<Mat3>& Fp, const std::vector<double>& m, const std::vector<double>& vol,
                   const std::vector<double>& rho, const std::vector<double>& q, double E, double nu, double thetaC,
                   double thetaS, double fr, uint8_t mat)
        : masses(m), volumes(vol), densities(rho), plasticAmount(q), velocities(v), positions(x),
          elasticDeformationGradients(Fe), plasticDeformationGradients(Fp), youngsModulus(E), poissonRatio(nu),
          criticalCompression(thetaC), criticalStretch(thetaS), friction(fr) {
        const size_t n = x.rows();
        if (v.rows() != n || Fe.size() != n || Fp.size() != n || m.size() != n || vol.size() != n ||
            rho.size() != n || q.size() != n)
            throw Error(AEP_INVALID_ARG, "ParticleSystem: inconsistent sizes");
        affineMomenta_1.resize(n);
        affineMomenta_2.resize(n);
        affineMomenta_3.resize(n);
        material.assign(n, mat);
    }
    size_t size() const { return positions.rows(); }

    // Seeded factories with the sampling, mass and material rules of the reference
    // (ParticleSystem.cpp:119-401): rejection sampling of the unit ball / disk,
    // total mass spread evenly, volumes 1 (the first P2G of solve recomputes them),
    // F_E = F_P = I.
    static ParticleSystem SnowBall(const Vec3& center, double radius, int n, uint64_t seed = 0) {
        return ball(center, radius, n, seed, 100.0, AEP_SNOW, 1.4e5, 0.2);
    }
    static ParticleSystem SandBall(const Vec3& center, double radius, int n, uint64_t seed = 0) {
        return ball(center, radius, n, seed, 1300.0, AEP_SAND, 3.537e5, 0.3);
    }
    // box minus a sphere of holeRadius centred at (bmin.x, bmin.y, mid z) (:261-329)
    static ParticleSystem SandBlock(const Vec3& bmin, const Vec3& bmax, double holeRadius, int n,
                                    uint64_t seed = 0) {
        if (holeRadius * 2.0 >= bmax[2] - bmin[2]) throw Error(AEP_INVALID_ARG, "SandBlock: the hole is too big");
        const Vec3 hc{bmin[0], bmin[1], 0.5 * (bmax[2] + bmin[2])};
        std::mt19937_64 g(seed);
        std::uniform_real_distribution<double> dx(bmin[0], bmax[0]), dy(bmin[1], bmax[1]), dz(bmin[2], bmax[2]);
        Block3<double> x((size_t)n);
        for (int i = 0; i < n;) {
            const Vec3 p{dx(g), dy(g), dz(g)};
            if (detail::norm(detail::sub(p, hc)) >= holeRadius) x.setRow((size_t)i++, p);
        }
        const double total = 1300.0 * ((bmax[0] - bmin[0]) * (bmax[1] - bmin[1]) * (bmax[2] - bmin[2]) -
                                       0.25 * detail::kPi * holeRadius * holeRadius * holeRadius);
        return make(x, Block3<double>((size_t)n), total, AEP_SAND, 3.537e5, 0.3);
    }
    // cylinder on baseCenter along +z, falling at 1 m/s (:331-401)
    static ParticleSystem SandCylinder(const Vec3& base, double radius, double height, int n, uint64_t seed = 0) {
        std::mt19937_64 g(seed);
        std::uniform_real_distribution<double> u(-1.0, 1.0), dz(0.0, height);
        Block3<double> x((size_t)n), v((size_t)n);
        for (int i = 0; i < n; ++i) {
            double a, b;
            do {
                a = u(g);
                b = u(g);
            } while (a * a + b * b > 1.0);
            x.setRow((size_t)i, {base[0] + radius * a, base[1] + radius * b, base[2] + dz(g)});
            v(i, 2) = -1.0;
        }
        return make(x, v, 1300.0 * detail::kPi * radius * radius * height, AEP_SAND, 3.537e5, 0.3);
    }

private:
    static ParticleSystem ball(const Vec3& c, double r, int n, uint64_t seed, double density, uint8_t mat, double E,
                               double nu) {
        std::mt19937_64 g(seed);
        std::uniform_real_distribution<double> u(-1.0, 1.0);
        Block3<double> x((size_t)n);
        for (int i = 0; i < n; ++i) {
            Vec3 p;
            do {
                p = {u(g), u(g), u(g)};
            } while (detail::norm(p) > 1.0);
            x.setRow((size_t)i, {c[0] + r * p[0], c[1] + r * p[1], c[2] + r * p[2]});
        }
        return make(x, Block3<double>((size_t)n), density * 3.14 * r * r * r, mat, E, nu);
    }
    static ParticleSystem make(const Block3<double>& x, const Block3<double>& v, double total, uint8_t mat, double E,
                               double nu) {
        const size_t n = x.rows();
        return ParticleSystem(v, x, std::vector<Mat3>(n, identity3()), std::vector<Mat3>(n, identity3()),
                              std::vector<double>(n, total / (double)n), std::vector<double>(n, 1.0),
                              std::vector<double>(n, 1.0), std::vector<double>(n, 0.0), E, nu, 2.5e-2, 7.5e-3, 0.2,
                              mat);
    }
};

// ------------------------------------------------------------------------------------
// LagrangianMesh (LagrangianMesh.h:12-116, LagrangianMesh.cpp:127-475)
class LagrangianMesh {
public:
    Block3<double> vertexPositions, vertexVelocities, elementPositions, elementVelocities;
    Block3<int32_t> faces;
    std::vector<double> vertexMasses, vertexVolumes, elementMasses, elementVolumes;
    Block3<double> elementDirections_1, elementDirections_2, elementDirections_3;
    Block3<double> elementRestDirections_1, elementRestDirections_2, elementRestDirections_3;
    Block3<double> vertexAffineMomenta_1, vertexAffineMomenta_2, vertexAffineMomenta_3;
    Block3<double> elementAffineMomenta_1, elementAffineMomenta_2, elementAffineMomenta_3;
    double mu = 0, lambda = 0, shearStiffness = 0, stiffness = 0, frictionCoeff = 0;

    LagrangianMesh() = default;
    // LagrangianMesh(V, F, vv, ve, mv, volv, me, vole, d1..3, drest1..3, mu, lambda,
    // shearStiffness, stiffness, frictionCoeff) (:127-195): element positions start
    // at the vertex centroids (:186-187)
    LagrangianMesh(const Block3<double>& V, const Block3<int32_t>& F, const Block3<double>& vv,
                   const Block3<double>& ve, const std::vector<double>& mv, const std::vector<double>& volv,
                   const std::vector<double>& me, const std::vector<double>& vole, const Block3<double>& d1,
                   const Block3<double>& d2, const Block3<double>& d3, const Block3<double>& dr1,
                   const Block3<double>& dr2, const Block3<double>& dr3, double mu_, double lambda_, double shear,
                   double stiff, double fric)
        : vertexPositions(V), vertexVelocities(vv), elementVelocities(ve), faces(F), vertexMasses(mv),
          vertexVolumes(volv), elementMasses(me), elementVolumes(vole), elementDirections_1(d1),
          elementDirections_2(d2), elementDirections_3(d3), elementRestDirections_1(dr1),
          elementRestDirections_2(dr2), elementRestDirections_3(dr3), mu(mu_), lambda(lambda_),
          shearStiffness(shear), stiffness(stiff), frictionCoeff(fric) {
        const size_t nv = V.rows(), nf = F.rows();
        if (vv.rows() != nv || ve.rows() != nf || mv.size() != nv || volv.size() != nv || me.size() != nf ||
            vole.size() != nf || d1.rows() != nf || d2.rows() != nf || d3.rows() != nf || dr1.rows() != nf ||
            dr2.rows() != nf || dr3.rows() != nf)
            throw Error(AEP_INVALID_ARG, "LagrangianMesh: inconsistent sizes");
        for (size_t f = 0; f < nf; ++f)
            for (int c = 0; c < 3; ++c)
                if (F(f, c) < 0 || (size_t)F(f, c) >= nv) throw Error(AEP_INVALID_ARG, "LagrangianMesh: bad face");
        vertexAffineMomenta_1.resize(nv);
        vertexAffineMomenta_2.resize(nv);
        vertexAffineMomenta_3.resize(nv);
        elementAffineMomenta_1.resize(nf);
        elementAffineMomenta_2.resize(nf);
        elementAffineMomenta_3.resize(nf);
        elementPositions.resize(nf);
        updateElementPositions();
    }

    size_t vertexNumber() const { return vertexPositions.rows(); }
    size_t elementNumber() const { return faces.rows(); }

    // updateElementPositions: centroid of the three vertices (:371-380)
    void updateElementPositions() {
        for (size_t f = 0; f < faces.rows(); ++f)
            for (int a = 0; a < 3; ++a)
                elementPositions(f, a) =
                    (vertexPositions(faces(f, 0), a) + vertexPositions(faces(f, 1), a) + vertexPositions(faces(f, 2), a)) /
                    3.0;
    }

    // bindConstraints (:354-363): the vector is read when the mesh is uploaded
    void bindConstraints(std::vector<double>* vertexIsFixed) {
        if (vertexIsFixed && vertexIsFixed->size() != vertexNumber())
            throw Error(AEP_INVALID_ARG, "bindConstraints: the constraints are not compatible");
        fixed_ = vertexIsFixed;
    }
    // vertexIsFixed (:462-475)
    bool vertexIsFixed(int v) const {
        if (!fixed_) return false;
        if (v < 0 || (size_t)v >= fixed_->size()) throw Error(AEP_INVALID_ARG, "vertexIsFixed: index out of range");
        return (*fixed_)[(size_t)v] != 0.0;
    }
    const std::vector<double>* constraints() const { return fixed_; }

    // Mesh from in-memory triangles with the rules of ObjMesh (:197-352): element
    // volume = area * thickness / 4, each vertex gets the volumes of its elements,
    // masses = density * volumes, rest directions (v2 - v1, v3 - v1, unit normal),
    // current directions = rest, Lame parameters from (E, nu), friction cap
    // tan(frictionAngleInDegree).
    static LagrangianMesh fromTriangles(const Block3<double>& V, const Block3<int32_t>& F, double density,
                                        double thickness, double E, double nu, double shear, double stiff,
                                        double frictionAngleInDegree) {
        const size_t nv = V.rows(), nf = F.rows();
        std::vector<double> volv(nv, 0.0), vole(nf, 0.0);
        Block3<double> d1(nf), d2(nf), d3(nf);
        for (size_t f = 0; f < nf; ++f) {
            for (int c = 0; c < 3; ++c)
                if (F(f, c) < 0 || (size_t)F(f, c) >= nv) throw Error(AEP_INVALID_ARG, "ObjMesh: face index out of range");
            const Vec3 v1 = V.row(F(f, 0)), v2 = V.row(F(f, 1)), v3 = V.row(F(f, 2));
            const double vol = 0.25 * detail::triangle_area(v1, v2, v3) * thickness;
            vole[f] = vol;
            for (int c = 0; c < 3; ++c) volv[F(f, c)] += vol;
            d1.setRow(f, detail::sub(v2, v1));
            d2.setRow(f, detail::sub(v3, v1));
            d3.setRow(f, detail::triangle_normal(v1, v2, v3));
        }
        std::vector<double> mv(nv), me(nf);
        for (size_t i = 0; i < nv; ++i) mv[i] = density * volv[i];
        for (size_t f = 0; f < nf; ++f) me[f] = density * vole[f];
        const double lambda = E * nu / (1.0 + nu) / (1.0 - 2.0 * nu), mu = E / 2.0 / (1.0 + nu);
        return LagrangianMesh(V, F, Block3<double>(nv), Block3<double>(nf), mv, volv, me, vole, d1, d2, d3, d1, d2, d3,
                              mu, lambda, shear, stiff, std::tan(frictionAngleInDegree * detail::kPi / 180.0));
    }

    // ObjMesh (:197-352): "v x y z" (read as float, as the reference does), "f a b c"
    // (1-based; a "a/b/c" token keeps its first index; 32-bit indices), other
    // records skipped to the end of the line.
    static LagrangianMesh ObjMesh(const std::string& filename, double density, double thickness, double E, double nu,
                                  double shear, double stiff, double frictionAngleInDegree) {
        std::ifstream in(filename);
        if (!in.is_open()) throw Error(AEP_INVALID_ARG, "ObjMesh: cannot open " + filename);
        std::vector<double> pos;
        std::vector<int64_t> idx;
        std::string mark, line;
        while (in >> mark) {
            if (mark == "v") {
                float p[3];
                if (!(in >> p[0] >> p[1] >> p[2])) throw Error(AEP_INVALID_ARG, "ObjMesh: bad vertex record");
                for (int a = 0; a < 3; ++a) pos.push_back((double)p[a]);
            } else if (mark == "f") {
                for (int c = 0; c < 3; ++c) {
                    std::string tok;
                    if (!(in >> tok)) throw Error(AEP_INVALID_ARG, "ObjMesh: bad face record");
                    idx.push_back(std::stoll(tok.substr(0, tok.find('/'))));
                }
            }
            std::getline(in, line);  // rest of the record (extra face vertices are not supported)
        }
        const size_t nv = pos.size() / 3, nf = idx.size() / 3;
        Block3<double> V(nv);
        Block3<int32_t> F(nf);
        for (size_t i = 0; i < nv; ++i) V.setRow(i, {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]});
        for (size_t f = 0; f < nf; ++f)
            for (int c = 0; c < 3; ++c) {
                const int64_t k = idx[3 * f + c] - 1;
                if (k < 0 || (size_t)k >= nv) throw Error(AEP_INVALID_ARG, "ObjMesh: face index out of range");
                F(f, c) = (int32_t)k;
            }
        return fromTriangles(V, F, density, thickness, E, nu, shear, stiff, frictionAngleInDegree);
    }

private:
    std::vector<double>* fixed_ = nullptr;
};

// ------------------------------------------------------------------------------------
// LevelSet (LevelSet.cpp:8-42): a union of analytic shapes in place of the
// std::function pair (phi, dphi) of HybridSolver::setLevelSet
class LevelSet {
public:
    std::vector<aep_sdf> shapes;
    static LevelSet plane(const Vec3& normal, double offset) {
        const double l = detail::norm(normal);
        return one(AEP_SDF_PLANE, {normal[0] / l, normal[1] / l, normal[2] / l, offset, 0, 0});
    }
    static LevelSet ground(double groundZ) { return plane({0, 0, 1}, groundZ); }  // groundLevelSet
    static LevelSet sphere(const Vec3& c, double r) { return one(AEP_SDF_SPHERE, {c[0], c[1], c[2], r, 0, 0}); }
    static LevelSet wall2ground(double wallX, double wallY, double groundZ) {  // wall2groundLevelSet
        return one(AEP_SDF_WALL2GROUND, {wallX, wallY, groundZ, 0, 0, 0});
    }
    LevelSet operator|(const LevelSet& o) const {
        LevelSet r = *this;
        r.shapes.insert(r.shapes.end(), o.shapes.begin(), o.shapes.end());
        return r;
    }

private:
    static LevelSet one(int32_t type, const std::array<double, 6>& p) {
        LevelSet l;
        aep_sdf s{};
        s.type = type;
        for (int k = 0; k < 6; ++k) s.p[k] = p[k];
        l.shapes.push_back(s);
        return l;
    }
};

// OBJ frame files of HybridSolver::solve (HybridSolver.cpp:991-1030): "v x y z"
// per point, faces "f a b c" 1-based, default stream formatting
inline void writeParticleObj(const std::string& path, const Block3<double>& x) {
    std::ofstream out(path);
    if (!out) throw Error(AEP_INVALID_ARG, "cannot write " + path);
    for (size_t p = 0; p < x.rows(); ++p) out << "v " << x(p, 0) << ' ' << x(p, 1) << ' ' << x(p, 2) << '\n';
}
inline void writeMeshObj(const std::string& path, const LagrangianMesh& m) {
    std::ofstream out(path);
    if (!out) throw Error(AEP_INVALID_ARG, "cannot write " + path);
    const Block3<double>& x = m.vertexPositions;
    for (size_t p = 0; p < x.rows(); ++p) out << "v " << x(p, 0) << ' ' << x(p, 1) << ' ' << x(p, 2) << '\n';
    for (size_t f = 0; f < m.faces.rows(); ++f)
        out << "f " << m.faces(f, 0) + 1 << ' ' << m.faces(f, 1) + 1 << ' ' << m.faces(f, 2) + 1 << '\n';
}

// ------------------------------------------------------------------------------------
// HybridSolver (HybridSolver.h:27-93) on the GPU
class HybridSolver {
public:
    struct WeightRow {  // one row of omegas_ / domegas_1..3 (HybridSolver.cpp:18-97)
        std::array<int64_t, 64> node;  // reference node index, -1: no node
        std::array<double, 64> w;
        std::array<Vec3, 64> grad;
    };

    explicit HybridSolver(ParticleSystem* ps = nullptr, RegularGrid* rg = nullptr) : ps_(ps), rg_(rg) {
        aep_default_params(&prm_);
    }
    ~HybridSolver() {
        if (h_) aep_solver_destroy(h_);
    }
    HybridSolver(const HybridSolver&) = delete;
    HybridSolver& operator=(const HybridSolver&) = delete;

    void setParticleSystem(ParticleSystem* ps) { ps_ = ps; dirty_ = true; }
    void setRegularGrid(RegularGrid* rg) {
        rg_ = rg;
        if (h_) {
            aep_solver_destroy(h_);
            h_ = nullptr;
        }
        dirty_ = true;
    }
    void setLagrangianMesh(LagrangianMesh* mesh) { mesh_ = mesh; dirty_ = true; }
    void setLevelSet(const LevelSet& ls) {
        ls_ = ls;
        if (h_) check(aep_set_levelset(h_, ls_.shapes.data(), (int32_t)ls_.shapes.size()), h_, "setLevelSet");
    }
    // Material and solver parameters.  By default the elastic constants come from
    // the bound ParticleSystem (its youngsModulus / poissonRatio, and for snow its
    // critical compression / stretch), as computeGridForces_ and updatePlasticity_
    // read them (HybridSolver.cpp:261-262, 626-631).
    void setParams(const aep_params& p) { prm_ = p; user_params_ = true; dirty_ = true; }
    const aep_params& params() const { return prm_; }
    // solve(): write the reference's frame files under this directory (empty: none)
    void setOutputDirectory(const std::string& dir) { out_dir_ = dir; }
    // solve(): called after each completed frame with (frame number, t); return
    // false to stop
    void setFrameCallback(std::function<bool(int, double)> fn) { frame_fn_ = std::move(fn); }

    // upload the bound objects now (otherwise done by the first step / solve)
    void push() {
        if (!rg_) throw Error(AEP_NOT_READY, "HybridSolver: no RegularGrid");
        if (!h_) {
            aep_grid_desc g = rg_->desc();
            apply_material();
            check(aep_solver_create(&g, &prm_, &h_), nullptr, "aep_solver_create");
        } else {
            apply_material();
            aep_solver* fresh = nullptr;  // parameters are fixed at creation
            aep_grid_desc g = rg_->desc();
            check(aep_solver_create(&g, &prm_, &fresh), nullptr, "aep_solver_create");
            aep_solver_destroy(h_);
            h_ = fresh;
        }
        check(aep_set_levelset(h_, ls_.shapes.data(), (int32_t)ls_.shapes.size()), h_, "aep_set_levelset");
        if (ps_ && ps_->size() > 0) {
            const size_t n = ps_->size();
            std::vector<double> B(9 * n), Fe(9 * n), Fp(9 * n), q(n);
            for (size_t i = 0; i < 3 * n; ++i) {
                B[i] = ps_->affineMomenta_1.data()[i];
                B[3 * n + i] = ps_->affineMomenta_2.data()[i];
                B[6 * n + i] = ps_->affineMomenta_3.data()[i];
            }
            for (size_t p = 0; p < n; ++p)
                for (int k = 0; k < 9; ++k) {
                    Fe[9 * p + k] = ps_->elasticDeformationGradients[p][k];
                    Fp[9 * p + k] = ps_->plasticDeformationGradients[p][k];
                }
            check(aep_set_particles(h_, (int64_t)n, ps_->positions.data(), ps_->velocities.data(), B.data(), Fe.data(),
                                    Fp.data(), ps_->masses.data(), ps_->volumes.data(), ps_->plasticAmount.data(),
                                    ps_->material.data()),
                  h_, "aep_set_particles");
        }
        if (mesh_) {
            LagrangianMesh& m = *mesh_;
            const size_t nf = m.elementNumber();
            std::vector<double> d(9 * nf), dr(9 * nf);
            for (size_t i = 0; i < 3 * nf; ++i) {
                d[i] = m.elementDirections_1.data()[i];
                d[3 * nf + i] = m.elementDirections_2.data()[i];
                d[6 * nf + i] = m.elementDirections_3.data()[i];
                dr[i] = m.elementRestDirections_1.data()[i];
                dr[3 * nf + i] = m.elementRestDirections_2.data()[i];
                dr[6 * nf + i] = m.elementRestDirections_3.data()[i];
            }
            check(aep_set_mesh(h_, (int64_t)m.vertexNumber(), (int64_t)nf, m.vertexPositions.data(), m.faces.data(),
                               m.vertexVelocities.data(), m.elementVelocities.data(), m.vertexMasses.data(),
                               m.vertexVolumes.data(), m.elementMasses.data(), m.elementVolumes.data(), d.data(),
                               dr.data(), m.mu, m.lambda, m.shearStiffness, m.stiffness, m.frictionCoeff),
                  h_, "aep_set_mesh");
            if (m.constraints())
                check(aep_set_fixed_vertices(h_, (int64_t)m.vertexNumber(), m.constraints()->data()), h_,
                      "aep_set_fixed_vertices");
        }
        dirty_ = false;
    }

    // first P2G with densities and volumes (HybridSolver.cpp:242-249, :854)
    void initVolumes() {
        ensure();
        check(aep_init_volumes(h_), h_, "aep_init_volumes");
    }
    // one loop body of solve with a fixed Dt (stream-ordered; pull() to read)
    void step(double dt) {
        ensure();
        check(aep_step(h_, dt), h_, "aep_step");
    }
    // the loop body with the reference's two Dts (force pass / grid update, the rest)
    void step(double dtForce, double dt) {
        ensure();
        check(aep_step_split(h_, dtForce, dt), h_, "aep_step_split");
    }

    // HybridSolver::solve(CFL, maxt, alpha) (HybridSolver.cpp:827-989): pulls the
    // state into the bound objects at every frame (and writes the frame files
    // when an output directory is set) and at the end
    void solve(double CFL, double maxt, double alpha) {
        ensure();
        frame_no_ = 0;
        if (!out_dir_.empty()) {
            detail::make_dirs(out_dir_);
            detail::make_dirs(out_dir_ + "/particle");
            detail::make_dirs(out_dir_ + "/mesh");
        }
        check(aep_set_solve_callback(h_, &HybridSolver::on_step, this), h_, "aep_set_solve_callback");
        aep_status st = aep_solve(h_, CFL, maxt, alpha);
        aep_set_solve_callback(h_, nullptr, nullptr);
        if (cb_error_) {
            cb_error_ = false;
            throw Error(AEP_INVALID_ARG, cb_what_);
        }
        check(st, h_, "aep_solve");
        pull();
    }
    aep_solve_state solveState() const {
        aep_solve_state s{};
        if (h_) aep_get_solve_state(h_, &s);
        return s;
    }

    // device state -> the bound ParticleSystem / LagrangianMesh members
    void pull() {
        if (!h_) return;
        if (ps_ && ps_->size() > 0) {
            const size_t n = ps_->size();
            std::vector<double> B(9 * n), Fe(9 * n), Fp, q(n), vol(n);
            if (prm_.track_plastic_F) Fp.resize(9 * n);
            check(aep_get_particles(h_, (int64_t)n, ps_->positions.data(), ps_->velocities.data(), B.data(), Fe.data(),
                                    prm_.track_plastic_F ? Fp.data() : nullptr, vol.data(), q.data()),
                  h_, "aep_get_particles");
            for (size_t i = 0; i < 3 * n; ++i) {
                ps_->affineMomenta_1.data()[i] = B[i];
                ps_->affineMomenta_2.data()[i] = B[3 * n + i];
                ps_->affineMomenta_3.data()[i] = B[6 * n + i];
            }
            for (size_t p = 0; p < n; ++p) {
                for (int k = 0; k < 9; ++k) {
                    ps_->elasticDeformationGradients[p][k] = Fe[9 * p + k];
                    if (prm_.track_plastic_F) ps_->plasticDeformationGradients[p][k] = Fp[9 * p + k];
                }
                ps_->volumes[p] = vol[p];
                if (ps_->material[p] == AEP_SAND) ps_->plasticAmount[p] = q[p];
                if (ps_->volumes[p] > 0.0) ps_->densities[p] = ps_->masses[p] / ps_->volumes[p];
            }
        }
        if (mesh_) {
            LagrangianMesh& m = *mesh_;
            const size_t nv = m.vertexNumber(), nf = m.elementNumber();
            std::vector<double> Bv(9 * nv), Be(9 * nf), d(9 * nf);
            check(aep_get_mesh(h_, m.vertexPositions.data(), m.vertexVelocities.data(), Bv.data(),
                               m.elementPositions.data(), m.elementVelocities.data(), Be.data(), d.data()),
                  h_, "aep_get_mesh");
            for (size_t i = 0; i < 3 * nv; ++i) {
                m.vertexAffineMomenta_1.data()[i] = Bv[i];
                m.vertexAffineMomenta_2.data()[i] = Bv[3 * nv + i];
                m.vertexAffineMomenta_3.data()[i] = Bv[6 * nv + i];
            }
            for (size_t i = 0; i < 3 * nf; ++i) {
                m.elementAffineMomenta_1.data()[i] = Be[i];
                m.elementAffineMomenta_2.data()[i] = Be[3 * nf + i];
                m.elementAffineMomenta_3.data()[i] = Be[6 * nf + i];
                m.elementDirections_1.data()[i] = d[i];
                m.elementDirections_2.data()[i] = d[3 * nf + i];
                m.elementDirections_3.data()[i] = d[6 * nf + i];
            }
        }
    }
    // device grid -> the bound RegularGrid's masses and velocities
    void pullGrid() {
        if (!h_ || !rg_) return;
        check(aep_get_grid(h_, rg_->masses.data(), rg_->velocities.data(), nullptr, nullptr), h_, "aep_get_grid");
    }

    // interpolation weights of item `item` (particles, then mesh vertices, then elements)
    WeightRow weights(int64_t item) {
        ensure();
        WeightRow r;
        std::array<double, 192> g;
        check(aep_get_weights(h_, 1, &item, r.node.data(), r.w.data(), g.data()), h_, "aep_get_weights");
        for (int k = 0; k < 64; ++k) r.grad[k] = {g[3 * k], g[3 * k + 1], g[3 * k + 2]};
        return r;
    }

    // full device state to / from a file (bit-exact resume)
    void saveCheckpoint(const std::string& path) {
        ensure();
        int64_t n = 0;
        check(aep_checkpoint_size(h_, &n), h_, "aep_checkpoint_size");
        std::vector<char> buf((size_t)n);
        check(aep_checkpoint_save(h_, buf.data(), n), h_, "aep_checkpoint_save");
        std::ofstream out(path, std::ios::binary);
        out.write(buf.data(), (std::streamsize)n);
        if (!out) throw Error(AEP_INVALID_ARG, "cannot write " + path);
    }
    void loadCheckpoint(const std::string& path) {
        std::ifstream in(path, std::ios::binary);
        if (!in) throw Error(AEP_INVALID_ARG, "cannot read " + path);
        std::vector<char> buf((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
        if (!h_) {
            if (!rg_) throw Error(AEP_NOT_READY, "HybridSolver: no RegularGrid");
            aep_grid_desc g = rg_->desc();
            check(aep_solver_create(&g, &prm_, &h_), nullptr, "aep_solver_create");
        }
        check(aep_checkpoint_load(h_, buf.data(), (int64_t)buf.size()), h_, "aep_checkpoint_load");
        dirty_ = false;
    }

    aep_stats stats() const {
        aep_stats s{};
        if (h_) aep_get_stats(h_, &s);
        return s;
    }
    aep_solver* handle() { return h_; }

private:
    void ensure() {
        if (dirty_ || !h_) push();
    }
    void apply_material() {
        if (user_params_ || !ps_ || ps_->size() == 0) return;
        bool snow = false, sand = false;
        for (uint8_t m : ps_->material) (m == AEP_SNOW ? snow : sand) = true;
        if (snow) {
            prm_.snow.E = ps_->youngsModulus;
            prm_.snow.nu = ps_->poissonRatio;
            prm_.snow.theta_c = ps_->criticalCompression;
            prm_.snow.theta_s = ps_->criticalStretch;
        }
        if (sand) {
            prm_.sand.E = ps_->youngsModulus;
            prm_.sand.nu = ps_->poissonRatio;
        }
    }
    static int32_t on_step(aep_solver*, const aep_solve_state* st, void* user) {
        HybridSolver* self = static_cast<HybridSolver*>(user);
        if (!st->frame_done) return 0;
        try {
            const int frame = self->frame_no_++;
            if (!self->out_dir_.empty()) {
                std::ostringstream ss;
                ss << frame;
                if (self->ps_ && self->ps_->size() > 0) {
                    check(aep_get_particles(self->h_, (int64_t)self->ps_->size(), self->ps_->positions.data(), nullptr,
                                            nullptr, nullptr, nullptr, nullptr, nullptr),
                          self->h_, "aep_get_particles");
                    writeParticleObj(self->out_dir_ + "/particle/particle_" + ss.str() + ".obj", self->ps_->positions);
                }
                if (self->mesh_) {
                    check(aep_get_mesh(self->h_, self->mesh_->vertexPositions.data(), nullptr, nullptr, nullptr,
                                       nullptr, nullptr, nullptr),
                          self->h_, "aep_get_mesh");
                    writeMeshObj(self->out_dir_ + "/mesh/mesh_" + ss.str() + ".obj", *self->mesh_);
                }
            }
            if (self->frame_fn_ && !self->frame_fn_(frame, st->t)) return 1;
        } catch (const std::exception& e) {  // exceptions cannot cross the C frame
            self->cb_error_ = true;
            self->cb_what_ = e.what();
            return 1;
        }
        return 0;
    }

    ParticleSystem* ps_ = nullptr;
    RegularGrid* rg_ = nullptr;
    LagrangianMesh* mesh_ = nullptr;
    LevelSet ls_;
    aep_params prm_{};
    bool user_params_ = false;
    bool dirty_ = true;
    aep_solver* h_ = nullptr;
    std::string out_dir_;
    std::function<bool(int, double)> frame_fn_;
    int frame_no_ = 0;
    bool cb_error_ = false;
    std::string cb_what_;
};

}  // namespace aep
