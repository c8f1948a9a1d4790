/*
 * aep_oracle.cpp -- FP64 CPU restatement of the reference MPM step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker, never the product:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * the library built from it.  The product path (libaep.so) never links it.
 *
 * What it restates (all citations relative to the reference project root,
 * AnisotropicElastoplasticity/):
 *   - weights           HybridSolver.cpp:18-97, interpolation.cpp:9-33
 *   - P2G (+ volumes)   HybridSolver.cpp:113-250
 *   - grid forces       HybridSolver.cpp:252-458, LagrangianMesh.cpp:382-460
 *   - collision         HybridSolver.cpp:460-511 (incl. the stray ';' at :500-501)
 *   - F update          HybridSolver.cpp:553-609
 *   - return mapping    HybridSolver.cpp:612-723
 *   - grid update       HybridSolver.cpp:725-737
 *   - G2P / APIC        HybridSolver.cpp:739-825
 *   - step order        HybridSolver.cpp:867-989
 *   - QR, inverseR      geometry.cpp:31-73;  level sets LevelSet.cpp:8-42
 * It keeps the reference dataflow: per-step sparse weight matrices (row-major
 * per particle plus the node-major transpose that Eigen's setFromTriplets
 * builds), two scatters and two gathers per step, two 3x3 SVDs per particle.
 *
 * Generalisations (each reduces to the reference when left at its default):
 * per-particle material tag instead of the hard-coded SAND of :873,955,959;
 * gravity vector instead of the literal -9.8 on axis 2 (:457); friction mu
 * instead of the literal 0.2 (:465); a union of level-set shapes instead of
 * one std::function pair.
 *
 * PARITY UNPINNED: the reference cannot be compiled in this environment (it
 * needs Eigen 3 and libigl, neither is present) and it ships no tests, no
 * fixtures and no golden vectors.  The 3x3 SVD is Eigen::JacobiSVD in the
 * reference (third-party, unpinned version); every quantity the step takes
 * from an SVD (U V^T, U f(S) V^T, V S^-1 U^T) is invariant under the SVD's
 * sign/order freedom, so this file's own one-sided Jacobi SVD reproduces it
 * to rounding.  This restatement is pinned only by mathematical known-answer
 * tests (tests/test_oracle_kat.py).
 */
#include "../include/aep.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double kPi = 3.14159265358979323846;  // igl::PI
typedef std::array<double, 3> V3;
typedef std::array<double, 9> M3;  // column-major: m[a + 3*b] = M(a, b)

inline double& E(M3& m, int a, int b) { return m[a + 3 * b]; }
inline double E(const M3& m, int a, int b) { return m[a + 3 * b]; }

M3 ident() { M3 m{}; m[0] = m[4] = m[8] = 1.0; return m; }
M3 mul(const M3& A, const M3& B) {
    M3 C{};
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            double s = 0;
            for (int k = 0; k < 3; ++k) s += E(A, a, k) * E(B, k, b);
            E(C, a, b) = s;
        }
    return C;
}
M3 transpose(const M3& A) {
    M3 T;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) E(T, a, b) = E(A, b, a);
    return T;
}
double det(const M3& A) {
    return E(A, 0, 0) * (E(A, 1, 1) * E(A, 2, 2) - E(A, 1, 2) * E(A, 2, 1))
         - E(A, 0, 1) * (E(A, 1, 0) * E(A, 2, 2) - E(A, 1, 2) * E(A, 2, 0))
         + E(A, 0, 2) * (E(A, 1, 0) * E(A, 2, 1) - E(A, 1, 1) * E(A, 2, 0));
}
// cofactor matrix: cof(A) = det(A) * A^-T
M3 cofactor(const M3& A) {
    M3 C;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            int a1 = (a + 1) % 3, a2 = (a + 2) % 3, b1 = (b + 1) % 3, b2 = (b + 2) % 3;
            E(C, a, b) = E(A, a1, b1) * E(A, a2, b2) - E(A, a1, b2) * E(A, a2, b1);
        }
    return C;
}
V3 matvec(const M3& A, const V3& x) {
    V3 y;
    for (int a = 0; a < 3; ++a) y[a] = E(A, a, 0) * x[0] + E(A, a, 1) * x[1] + E(A, a, 2) * x[2];
    return y;
}
double dot(const V3& a, const V3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
double norm(const V3& a) { return std::sqrt(dot(a, a)); }
V3 cross(const V3& a, const V3& b) {
    return V3{a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}

// ---- interpolation.cpp:9-33 (cubic B-spline and its derivative) -------------------
double cubic_B_spline(double x) {
    double ax = std::fabs(x);
    if (ax >= 2.0) return 0.0;
    if (ax >= 1.0) return -1.0 / 6.0 * ax * ax * ax + ax * ax - 2.0 * ax + 4.0 / 3.0;
    return 0.5 * ax * ax * ax - ax * ax + 2.0 / 3.0;
}
double Dcubic_B_spline(double x) {
    if (x >= 2.0) return 0.0;
    if (x >= 1.0) return -0.5 * x * x + 2.0 * x - 2.0;
    if (x >= 0.0) return 1.5 * x * x - 2.0 * x;
    if (x >= -1.0) return -1.5 * x * x - 2.0 * x;
    if (x >= -2.0) return 0.5 * x * x + 2.0 * x + 2.0;
    return 0.0;
}

// ---- 3x3 SVD: one-sided (Hestenes) Jacobi, run to FP64 convergence ------------------
// Contract of Eigen::JacobiSVD<Matrix3d>(A, ComputeFullU|ComputeFullV) as used at
// HybridSolver.cpp:308,620: A = U diag(s) V^T, U and V orthogonal, s >= 0, sorted
// descending.
void svd3(const M3& A, M3& U, V3& s, M3& V) {
    M3 W = A;
    V = ident();
    for (int sweep = 0; sweep < 60; ++sweep) {
        bool rotated = false;
        for (int pq = 0; pq < 3; ++pq) {
            int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
            double alpha = 0, beta = 0, gamma = 0;
            for (int r = 0; r < 3; ++r) {
                alpha += E(W, r, p) * E(W, r, p);
                beta += E(W, r, q) * E(W, r, q);
                gamma += E(W, r, p) * E(W, r, q);
            }
            if (std::fabs(gamma) <= 1e-16 * std::sqrt(alpha * beta) || gamma == 0.0) continue;
            rotated = true;
            double zeta = (beta - alpha) / (2.0 * gamma);
            double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
            double c = 1.0 / std::sqrt(1.0 + t * t), sn = c * t;
            for (int r = 0; r < 3; ++r) {
                double wp = E(W, r, p), wq = E(W, r, q);
                E(W, r, p) = c * wp - sn * wq;
                E(W, r, q) = sn * wp + c * wq;
                double vp = E(V, r, p), vq = E(V, r, q);
                E(V, r, p) = c * vp - sn * vq;
                E(V, r, q) = sn * vp + c * vq;
            }
        }
        if (!rotated) break;
    }
    V3 cn;
    for (int b = 0; b < 3; ++b)
        cn[b] = std::sqrt(E(W, 0, b) * E(W, 0, b) + E(W, 1, b) * E(W, 1, b) + E(W, 2, b) * E(W, 2, b));
    int order[3] = {0, 1, 2};
    std::sort(order, order + 3, [&](int a, int b) { return cn[a] > cn[b]; });
    M3 W2, V2;
    for (int b = 0; b < 3; ++b) {
        s[b] = cn[order[b]];
        for (int r = 0; r < 3; ++r) {
            E(W2, r, b) = E(W, r, order[b]);
            E(V2, r, b) = E(V, r, order[b]);
        }
    }
    V = V2;
    // U columns: normalised columns of A V; complete the basis where s is ~0.
    double tiny = 1e-300 + 1e-14 * s[0];
    for (int b = 0; b < 3; ++b) {
        if (s[b] > tiny) {
            for (int r = 0; r < 3; ++r) E(U, r, b) = E(W2, r, b) / s[b];
        } else {
            V3 u;
            if (b == 2 && s[1] > tiny) {
                V3 u0{E(U, 0, 0), E(U, 1, 0), E(U, 2, 0)}, u1{E(U, 0, 1), E(U, 1, 1), E(U, 2, 1)};
                u = cross(u0, u1);
            } else {
                // pick any unit vector orthogonal to the previous columns
                V3 e[3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
                for (int k = 0; k < 3; ++k) {
                    u = e[k];
                    for (int c = 0; c < b; ++c) {
                        V3 uc{E(U, 0, c), E(U, 1, c), E(U, 2, c)};
                        double d = dot(u, uc);
                        for (int r = 0; r < 3; ++r) u[r] -= d * uc[r];
                    }
                    if (norm(u) > 0.5) break;
                }
            }
            double nu = norm(u);
            for (int r = 0; r < 3; ++r) E(U, r, b) = u[r] / nu;
            s[b] = std::max(s[b], 0.0);
        }
    }
}

// ---- geometry.cpp:31-62 (classical Gram-Schmidt QR of [d1 d2 d3]) ---------------
void gram_schmidt(const M3& D, M3& Q, M3& R) {
    V3 d1{E(D, 0, 0), E(D, 1, 0), E(D, 2, 0)};
    V3 d2{E(D, 0, 1), E(D, 1, 1), E(D, 2, 1)};
    V3 d3{E(D, 0, 2), E(D, 1, 2), E(D, 2, 2)};
    double r11 = norm(d1);
    V3 q1{d1[0] / r11, d1[1] / r11, d1[2] / r11};
    double r12 = dot(d2, q1);
    V3 q2{d2[0] - r12 * q1[0], d2[1] - r12 * q1[1], d2[2] - r12 * q1[2]};
    double r22 = norm(q2);
    for (int r = 0; r < 3; ++r) q2[r] /= r22;
    double r13 = dot(d3, q1), r23 = dot(d3, q2);
    V3 q3{d3[0] - r13 * q1[0] - r23 * q2[0], d3[1] - r13 * q1[1] - r23 * q2[1],
          d3[2] - r13 * q1[2] - r23 * q2[2]};
    double r33 = norm(q3);
    for (int r = 0; r < 3; ++r) q3[r] /= r33;
    for (int r = 0; r < 3; ++r) {
        E(Q, r, 0) = q1[r];
        E(Q, r, 1) = q2[r];
        E(Q, r, 2) = q3[r];
    }
    R = M3{};
    E(R, 0, 0) = r11; E(R, 0, 1) = r12; E(R, 0, 2) = r13;
    E(R, 1, 1) = r22; E(R, 1, 2) = r23;
    E(R, 2, 2) = r33;
}

// 2x2 polar rotation U V^T of the SVD (Eigen::JacobiSVD<Matrix2d> at
// LagrangianMesh.cpp:437-438).  M(a,b) = m[a + 2b].
void polar2(const double m[4], double R[4]) {
    double a = m[0], c = m[1], b = m[2], d = m[3];
    double dt = a * d - b * c;
    if (dt >= 0) {
        double th = std::atan2(c - b, a + d);
        R[0] = std::cos(th); R[1] = std::sin(th); R[2] = -std::sin(th); R[3] = std::cos(th);
    } else {
        double ph = std::atan2(b + c, a - d);
        R[0] = std::cos(ph); R[1] = std::sin(ph); R[2] = std::sin(ph); R[3] = -std::cos(ph);
    }
}

// ---- level sets: LevelSet.cpp:8-42, unioned by min ---------------------------------
struct Shape { int type; double p[6]; };

void levelset(const std::vector<Shape>& shapes, const V3& x, double& phi, V3& n) {
    phi = INFINITY;
    n = V3{0, 0, 1};
    for (const Shape& s : shapes) {
        double ph;
        V3 nn;
        if (s.type == AEP_SDF_PLANE) {
            ph = s.p[0] * x[0] + s.p[1] * x[1] + s.p[2] * x[2] - s.p[3];
            nn = V3{s.p[0], s.p[1], s.p[2]};
        } else if (s.type == AEP_SDF_SPHERE) {
            V3 d{x[0] - s.p[0], x[1] - s.p[1], x[2] - s.p[2]};
            double r = norm(d);
            ph = r - s.p[3];
            nn = r > 0 ? V3{d[0] / r, d[1] / r, d[2] / r} : V3{0, 0, 1};
        } else {  // wall2groundLevelSet / Dwall2groundLevelSet
            double X = s.p[0], Y = s.p[1], G = s.p[2];
            ph = std::min(std::min(x[2] - G, X - x[0]), Y - x[1]);
            double dz = std::fabs(x[2] - G), dx = std::fabs(X - x[0]), dy = std::fabs(Y - x[1]);
            if (dz <= dx && dz <= dy) nn = V3{0, 0, 1};
            else if (dy <= dx) nn = V3{0, -1, 0};
            else nn = V3{-1, 0, 0};
        }
        if (ph < phi) { phi = ph; n = nn; }
    }
}

// ---- sparse weights (HybridSolver.cpp:18-97) ----------------------------------------
struct Grid {
    double min[3], h[3];
    int res[3];
    int64_t ng() const { return (int64_t)res[0] * res[1] * res[2]; }
    int64_t index(int i, int j, int k) const { return (int64_t)k * res[0] * res[1] + (int64_t)j * res[0] + i; }
    V3 node_pos(int64_t n) const {
        int64_t k = n / ((int64_t)res[0] * res[1]);
        int64_t j = (n % ((int64_t)res[0] * res[1])) / res[0];
        int64_t i = n - k * res[0] * res[1] - j * res[0];
        return V3{min[0] + i * h[0], min[1] + j * h[1], min[2] + k * h[2]};
    }
};

struct Weights {
    std::vector<int64_t> rowptr;
    std::vector<int64_t> node;
    std::vector<double> w, g0, g1, g2;
    std::vector<int64_t> colptr;  // node-major transpose (Eigen's column-major storage)
    std::vector<int64_t> colent;  // entry ids, ascending particle order within a column
    std::vector<int64_t> row;     // particle of each entry
    bool truncated_any = false;
};

template <class F>
void particle_stencil(const Grid& g, const V3& pos, F&& emit) {
    double pr[3] = {pos[0] - g.min[0], pos[1] - g.min[1], pos[2] - g.min[2]};
    int fl[3];
    for (int a = 0; a < 3; ++a) fl[a] = static_cast<int>(pr[a] / g.h[a]);  // truncation, as :34-36
    for (int i = fl[0] - 2; i <= fl[0] + 2; ++i)
        for (int j = fl[1] - 2; j <= fl[1] + 2; ++j)
            for (int k = fl[2] - 2; k <= fl[2] + 2; ++k) {
                if (!(0 <= i && i < g.res[0] && 0 <= j && j < g.res[1] && 0 <= k && k < g.res[2])) continue;
                double di = cubic_B_spline(pr[0] / g.h[0] - i);
                double dj = cubic_B_spline(pr[1] / g.h[1] - j);
                double dk = cubic_B_spline(pr[2] / g.h[2] - k);
                double ddi = Dcubic_B_spline(pr[0] / g.h[0] - i) / g.h[0];
                double ddj = Dcubic_B_spline(pr[1] / g.h[1] - j) / g.h[1];
                double ddk = Dcubic_B_spline(pr[2] / g.h[2] - k) / g.h[2];
                if (di > 0 && dj > 0 && dk > 0)
                    emit(g.index(i, j, k), di * dj * dk, ddi * dj * dk, di * ddj * dk, di * dj * ddk);
            }
}

void build_weights(const Grid& g, const std::vector<V3>& pos, Weights& W) {
    int64_t np = (int64_t)pos.size();
    W.rowptr.assign(np + 1, 0);
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < np; ++p) {
        int64_t c = 0;
        particle_stencil(g, pos[p], [&](int64_t, double, double, double, double) { ++c; });
        W.rowptr[p + 1] = c;
    }
    for (int64_t p = 0; p < np; ++p) W.rowptr[p + 1] += W.rowptr[p];
    int64_t nnz = W.rowptr[np];
    W.node.resize(nnz); W.w.resize(nnz); W.g0.resize(nnz); W.g1.resize(nnz); W.g2.resize(nnz);
    W.row.resize(nnz);
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < np; ++p) {
        int64_t e = W.rowptr[p];
        particle_stencil(g, pos[p], [&](int64_t n, double w, double a, double b, double c) {
            W.node[e] = n; W.w[e] = w; W.g0[e] = a; W.g1[e] = b; W.g2[e] = c; W.row[e] = p; ++e;
        });
    }
    // node-major transpose: a counting sort by node, stable in particle order
    int64_t ng = g.ng();
    W.colptr.assign(ng + 1, 0);
    for (int64_t e = 0; e < nnz; ++e) W.colptr[W.node[e] + 1]++;
    for (int64_t n = 0; n < ng; ++n) W.colptr[n + 1] += W.colptr[n];
    W.colent.resize(nnz);
    std::vector<int64_t> fill(W.colptr.begin(), W.colptr.end() - 1);
    for (int64_t e = 0; e < nnz; ++e) W.colent[fill[W.node[e]]++] = e;
}

// ---- solver state --------------------------------------------------------------------
struct Mesh {
    int64_t nv = 0, nf = 0;
    std::vector<V3> xv, vv, xe, ve;
    std::vector<M3> Bv, Be;  // 3x3 affine momenta (row a of B_p = affineMomenta_(a+1).row(p))
    std::vector<double> mv, volv, me, vole;
    std::vector<std::array<int, 3>> faces;
    std::vector<M3> D, Drest;  // columns d1 d2 d3
    double mu = 0, lambda = 0, shear = 0, stiffness = 0, friction = 0;
    std::vector<double> inplane;  // per element: 2x2 (invRest * P), column-major
    std::vector<uint8_t> fixed;   // LagrangianMesh::vertexIsFixed (LM:354-363, 462-475)
};

struct Oracle {
    Grid g;
    aep_params prm;
    std::vector<Shape> shapes;
    // particles
    int64_t np = 0;
    std::vector<V3> x, v;
    std::vector<M3> B, Fe, Fp, Fcand;
    std::vector<double> m, vol, rho, plastic;
    std::vector<uint8_t> mat;
    std::vector<M3> last_stress;
    Mesh mesh;
    bool has_mesh = false;
    // grid
    std::vector<double> gm;
    std::vector<V3> gv, gf, gvbf;
    Weights W, Wv, We;
    int64_t steps = 0;
};

void lame(double E_, double nu, double& lambda, double& mu) {
    lambda = E_ * nu / (1.0 + nu) / (1.0 - 2.0 * nu);
    mu = E_ / 2.0 / (1.0 + nu);
}

// scatter of one particle set into the grid (transposed products, node-parallel).
// fn(entry, particle) returns the contribution added to node value.
template <class T, class Fn>
void scatter(const Grid& g, const Weights& W, std::vector<T>& out, Fn&& fn) {
    int64_t ng = g.ng();
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t n = 0; n < ng; ++n) {
        for (int64_t s = W.colptr[n]; s < W.colptr[n + 1]; ++s) {
            int64_t e = W.colent[s];
            fn(out[n], e, W.row[e]);
        }
    }
}

// HybridSolver.cpp:113-250
void p2g_set(Oracle& o, const Weights& W, const std::vector<V3>& x, const std::vector<V3>& v,
             const std::vector<M3>& B, const std::vector<double>& m, std::vector<V3>& mom) {
    const Grid& g = o.g;
    double h = std::min(g.h[0], std::min(g.h[1], g.h[2]));
    double ratio = 3.0 / h / h;  // inertiaTensorRatio, :175-177
    int64_t ng = g.ng();
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t n = 0; n < ng; ++n) {
        if (W.colptr[n] == W.colptr[n + 1]) continue;
        V3 xn = g.node_pos(n);
        double ms = 0;
        V3 pm{0, 0, 0};
        for (int64_t s = W.colptr[n]; s < W.colptr[n + 1]; ++s) {
            int64_t e = W.colent[s], p = W.row[e];
            double w = W.w[e];
            ms += w * m[p];
            V3 dx{xn[0] - x[p][0], xn[1] - x[p][1], xn[2] - x[p][2]};
            V3 Bdx = matvec(B[p], dx);
            for (int a = 0; a < 3; ++a) pm[a] += w * m[p] * (v[p][a] + ratio * Bdx[a]);
        }
        o.gm[n] += ms;
        for (int a = 0; a < 3; ++a) mom[n][a] += pm[a];
    }
}

void p2g(Oracle& o, bool volumes) {
    int64_t ng = o.g.ng();
    o.gm.assign(ng, 0.0);
    std::vector<V3> mom(ng, V3{0, 0, 0});
    if (o.np) p2g_set(o, o.W, o.x, o.v, o.B, o.m, mom);
    if (o.has_mesh) {
        p2g_set(o, o.Wv, o.mesh.xv, o.mesh.vv, o.mesh.Bv, o.mesh.mv, mom);
        p2g_set(o, o.We, o.mesh.xe, o.mesh.ve, o.mesh.Be, o.mesh.me, mom);
    }
    o.gv.assign(ng, V3{0, 0, 0});
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < ng; ++n)
        if (o.gm[n] > 0.0)
            for (int a = 0; a < 3; ++a) o.gv[n][a] = mom[n][a] / o.gm[n];
    if (volumes && o.np) {  // :242-249
        double cellvol = o.g.h[0] * o.g.h[1] * o.g.h[2];
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < o.np; ++p) {
            double s = 0;
            for (int64_t e = o.W.rowptr[p]; e < o.W.rowptr[p + 1]; ++e) s += o.W.w[e] * o.gm[o.W.node[e]];
            o.rho[p] = s / cellvol;
            o.vol[p] = o.m[p] / o.rho[p];
        }
    }
}

// velocity gradient sum_i u_i (grad w_ip)^T of one particle (the three SpMVs of :269-271)
M3 grad_gather(const Weights& W, int64_t p, const std::vector<V3>& u) {
    M3 G{};
    for (int64_t e = W.rowptr[p]; e < W.rowptr[p + 1]; ++e) {
        const V3& un = u[W.node[e]];
        double gb[3] = {W.g0[e], W.g1[e], W.g2[e]};
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) E(G, a, b) += un[a] * gb[b];
    }
    return G;
}

// per-particle stress of :277-352 (returns the 3x3 "cauchyStress" incl. the volume)
M3 particle_stress(const Oracle& o, int64_t p, const M3& G, double dt) {
    const aep_params& P = o.prm;
    double lambda, mu;
    const M3& F = o.Fe[p];
    M3 Fh = F;
    M3 GF = mul(G, F);
    for (int k = 0; k < 9; ++k) Fh[k] += dt * GF[k];  // virtualEDG = EDG + EDG_modifier*EDG
    M3 U, V;
    V3 S;
    svd3(Fh, U, S, V);
    M3 st{};
    if (o.mat[p] == AEP_SNOW) {
        double l0, m0;
        lame(P.snow.E, P.snow.nu, l0, m0);
        double Jp = det(o.Fp[p]);  // :283, the oracle always keeps the full F_P
        double hard = std::exp(P.snow.xi * (1.0 - Jp));
        lambda = l0 * hard;
        mu = m0 * hard;
        M3 R = mul(U, transpose(V));
        double J = det(Fh);
        M3 C = cofactor(Fh);  // J * Fh^-T
        M3 A;
        for (int k = 0; k < 9; ++k) A[k] = 2.0 * mu * (Fh[k] - R[k]) + lambda * (J - 1.0) * C[k];
        st = mul(A, transpose(F));
    } else {
        lame(P.sand.E, P.sand.nu, lambda, mu);
        double lnS[3] = {std::log(S[0]), std::log(S[1]), std::log(S[2])};
        double tr = lnS[0] + lnS[1] + lnS[2];
        M3 Dg{};
        for (int a = 0; a < 3; ++a) E(Dg, a, a) = 2 * mu * (lnS[a] / S[a]) + lambda * tr / S[a];
        st = mul(mul(mul(U, Dg), transpose(V)), transpose(F));
    }
    for (int k = 0; k < 9; ++k) st[k] *= o.vol[p];
    return st;
}

// LagrangianMesh.cpp:382-460; returns vertex forces and stores invRest*P per element
void vertex_inplane_forces(Oracle& o, std::vector<V3>& fv) {
    Mesh& me = o.mesh;
    fv.assign(me.nv, V3{0, 0, 0});
    me.inplane.assign(4 * me.nf, 0.0);
    std::vector<std::array<V3, 3>> fe(me.nf);
#pragma omp parallel for schedule(static)
    for (int64_t f = 0; f < me.nf; ++f) {
        M3 Q, R, rQ, rR;
        gram_schmidt(me.D[f], Q, R);
        gram_schmidt(me.Drest[f], rQ, rR);
        // inverseR of the rest 2x2 block (geometry.cpp:67-73)
        double i11 = 1.0 / E(rR, 0, 0), i12 = -E(rR, 0, 1) / E(rR, 0, 0) / E(rR, 1, 1), i22 = 1.0 / E(rR, 1, 1);
        double r00 = E(R, 0, 0), r01 = E(R, 0, 1), r11 = E(R, 1, 1);
        // refInPlaneR = invRest * inPlaneR (upper triangular)
        double t00 = i11 * r00, t01 = i11 * r01 + i12 * r11, t11 = i22 * r11;
        double Rt[4] = {t00, 0.0, t01, t11};
        double rot[4];
        polar2(Rt, rot);
        double J = t00 * t11;
        // invRefMulDet^T = [[t11, 0], [-t01, t00]]
        double cofT[4] = {t11, -t01, 0.0, t00};
        double Pk[4];
        for (int k = 0; k < 4; ++k) Pk[k] = 2.0 * me.mu * (Rt[k] - rot[k]) + me.lambda * (J - 1.0) * cofT[k];
        // invRest * P  (invRest = [[i11, i12], [0, i22]])
        double* ip = &me.inplane[4 * f];
        ip[0] = i11 * Pk[0] + i12 * Pk[1];
        ip[1] = i22 * Pk[1];
        ip[2] = i11 * Pk[2] + i12 * Pk[3];
        ip[3] = i22 * Pk[3];
        double dr11 = Pk[0], dr12 = Pk[2], dr22 = Pk[3];
        V3 q1{E(Q, 0, 0), E(Q, 1, 0), E(Q, 2, 0)}, q2{E(Q, 0, 1), E(Q, 1, 1), E(Q, 2, 1)};
        V3 f2, f3, f1;
        // the reference does not weight these forces by the element volume; the
        // cloth_volume_weighting parameter (off by default) does
        double fw = o.prm.cloth_volume_weighting ? me.vole[f] : 1.0;
        for (int r = 0; r < 3; ++r) {
            f2[r] = -(dr11 * i11 + dr12 * i12) * q1[r] * fw;
            f3[r] = (-dr12 * i22 * q1[r] - dr22 * i22 * q2[r]) * fw;
            f1[r] = -(f2[r] + f3[r]);
        }
        fe[f] = {f1, f2, f3};
    }
    for (int64_t f = 0; f < me.nf; ++f)
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) fv[me.faces[f][c]][r] += fe[f][c][r];
}

// HybridSolver.cpp:389-442, the normal/shear stress of one element
M3 element_normal_stress(const Oracle& o, int64_t f) {
    const Mesh& me = o.mesh;
    M3 Q, R;
    gram_schmidt(me.D[f], Q, R);
    const double* ip = &me.inplane[4 * f];
    double dr11 = ip[0], dr12 = ip[2], dr22 = ip[3];
    double dr13 = me.shear * E(R, 0, 2), dr23 = me.shear * E(R, 1, 2);
    double r33 = E(R, 2, 2);
    double dr33 = r33 > 1.0 ? 0.0 : -me.stiffness * (1.0 - r33) * (1.0 - r33);
    M3 dR{};
    E(dR, 0, 0) = dr11; E(dR, 0, 1) = dr12; E(dR, 0, 2) = dr13;
    E(dR, 1, 1) = dr22; E(dR, 1, 2) = dr23; E(dR, 2, 2) = dr33;
    M3 K = mul(dR, transpose(R));
    M3 Ms;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) E(Ms, a, b) = a <= b ? E(K, a, b) : E(K, b, a);
    // R^-1 of the upper-triangular R
    M3 Ri{};
    double a00 = E(R, 0, 0), a01 = E(R, 0, 1), a02 = E(R, 0, 2), a11 = E(R, 1, 1), a12 = E(R, 1, 2), a22 = E(R, 2, 2);
    E(Ri, 0, 0) = 1.0 / a00;
    E(Ri, 1, 1) = 1.0 / a11;
    E(Ri, 2, 2) = 1.0 / a22;
    E(Ri, 0, 1) = -a01 / (a00 * a11);
    E(Ri, 1, 2) = -a12 / (a11 * a22);
    E(Ri, 0, 2) = (a01 * a12 - a02 * a11) / (a00 * a11 * a22);
    V3 wv{E(me.Drest[f], 2, 0), E(me.Drest[f], 2, 1), E(me.Drest[f], 2, 2)};  // (D_rest^T).col(2)
    V3 dF3 = matvec(Q, matvec(Ms, matvec(transpose(Ri), wv)));
    V3 d3{E(me.D[f], 0, 2), E(me.D[f], 1, 2), E(me.D[f], 2, 2)};
    M3 st;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) E(st, a, b) = me.vole[f] * dF3[a] * d3[b];
    return st;
}

// HybridSolver.cpp:252-458
void compute_forces(Oracle& o, double dt) {
    int64_t ng = o.g.ng();
    o.gf.assign(ng, V3{0, 0, 0});
    if (o.np) {
        o.last_stress.resize(o.np);
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < o.np; ++p) {
            M3 G = grad_gather(o.W, p, o.gv);
            o.last_stress[p] = particle_stress(o, p, G, dt);
        }
        const std::vector<M3>& st = o.last_stress;
        const Weights& W = o.W;
        scatter(o.g, W, o.gf, [&](V3& out, int64_t e, int64_t p) {
            double gb[3] = {W.g0[e], W.g1[e], W.g2[e]};
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) out[a] -= E(st[p], a, b) * gb[b];
        });
    }
    if (o.has_mesh) {
        std::vector<V3> fv;
        vertex_inplane_forces(o, fv);
        const Weights& Wv = o.Wv;
        scatter(o.g, Wv, o.gf, [&](V3& out, int64_t e, int64_t p) {
            for (int a = 0; a < 3; ++a) out[a] += Wv.w[e] * fv[p][a];
        });
        std::vector<M3> es(o.mesh.nf);
#pragma omp parallel for schedule(static)
        for (int64_t f = 0; f < o.mesh.nf; ++f) es[f] = element_normal_stress(o, f);
        const Weights& We = o.We;
        scatter(o.g, We, o.gf, [&](V3& out, int64_t e, int64_t f) {
            double gb[3] = {We.g0[e], We.g1[e], We.g2[e]};
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) out[a] -= E(es[f], a, b) * gb[b];
        });
    }
    // gravity (:457, generalised to a vector)
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < ng; ++n)
        for (int a = 0; a < 3; ++a) o.gf[n][a] += o.gm[n] * o.prm.gravity[a];
}

// HybridSolver.cpp:725-737
void update_grid_velocities(Oracle& o, double dt) {
    int64_t ng = o.g.ng();
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < ng; ++n)
        if (o.gm[n] > 0.0)
            for (int a = 0; a < 3; ++a) o.gv[n][a] += dt * o.gf[n][a] / o.gm[n];
}

// HybridSolver.cpp:513-550: every node of a fixed vertex's stencil zeroes the
// velocity and before-friction velocity of its 3x3x3 neighbours, addressed by the
// linear index k*Rx*Ry + j*Rx + i with the range check 0 <= index < Ng (i +- 1
// wraps into the next row, as in the reference; the distance test <= 12 always holds)
void fixed_vertices(Oracle& o) {
    if (!o.has_mesh || o.mesh.fixed.empty()) return;
    const Weights& W = o.Wv;
    const int64_t rx = o.g.res[0], ry = o.g.res[1], ng = o.g.ng();
    for (int64_t v = 0; v < o.mesh.nv; ++v) {
        if (!o.mesh.fixed[v]) continue;
        for (int64_t e = W.rowptr[v]; e < W.rowptr[v + 1]; ++e) {
            const int64_t node = W.node[e];
            const int64_t ri = node % rx, rj = (node / rx) % ry, rk = node / (rx * ry);
            for (int64_t i = ri - 1; i <= ri + 1; ++i)
                for (int64_t j = rj - 1; j <= rj + 1; ++j)
                    for (int64_t k = rk - 1; k <= rk + 1; ++k) {
                        const int64_t idx = k * rx * ry + j * rx + i;
                        if (0 <= idx && idx < ng) {
                            o.gv[idx] = V3{0, 0, 0};
                            o.gvbf[idx] = V3{0, 0, 0};
                        }
                    }
        }
    }
}

// HybridSolver.cpp:460-511, then the fixed-vertex sweep (:513-550)
void collision(Oracle& o) {
    int64_t ng = o.g.ng();
    o.gvbf = o.gv;
    double mu = o.prm.friction;
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < ng; ++n) {
        V3 xn = o.g.node_pos(n);
        double phi;
        V3 nrm;
        levelset(o.shapes, xn, phi, nrm);
        if (!(phi <= 0.0)) continue;
        V3 vr = o.gv[n];
        double vn = dot(vr, nrm);
        if (vn < 0.0) {
            V3 vt{vr[0] - vn * nrm[0], vr[1] - vn * nrm[1], vr[2] - vn * nrm[2]};
            o.gvbf[n] = vt;
            double nt = norm(vt);
            if (nt < -mu * vn) {
                vr = V3{0, 0, 0};
            } else if (o.prm.friction_bug) {
                vr = vt;  // the Coulomb decrement of :501 is a dead statement
            } else {
                for (int a = 0; a < 3; ++a) vr[a] = vt[a] + mu * vn * vt[a] / nt;
            }
            o.gv[n] = vr;
        }
    }
    fixed_vertices(o);
}

// G2P velocity, APIC (:739-825), advection (:940-951) for one particle set
void g2p_set(Oracle& o, const Weights& W, std::vector<V3>& x, std::vector<V3>& v, std::vector<M3>& B,
             double damp, double dt, bool advect, bool set_v) {
    int64_t n = (int64_t)x.size();
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < n; ++p) {
        V3 vp{0, 0, 0}, xp{0, 0, 0};
        M3 C{};
        for (int64_t e = W.rowptr[p]; e < W.rowptr[p + 1]; ++e) {
            int64_t nd = W.node[e];
            double w = W.w[e];
            V3 xn = o.g.node_pos(nd);
            const V3& vn = o.gv[nd];
            for (int a = 0; a < 3; ++a) {
                vp[a] += w * vn[a];
                for (int b = 0; b < 3; ++b) E(C, a, b) += w * vn[a] * (xn[b] - x[p][b]);
                xp[a] += w * (xn[a] + dt * o.gvbf[nd][a]);
            }
        }
        // damping of the symmetric part (:808-824)
        M3 Bn;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                double sym = 0.5 * (E(C, a, b) + E(C, b, a));
                E(Bn, a, b) = (E(C, a, b) - sym) + (1.0 - damp) * sym;
            }
        B[p] = Bn;
        if (set_v) v[p] = vp;
        if (advect) x[p] = xp;
    }
}

// singular-value return mapping, HybridSolver.cpp:626-674 (snow clamp, sand
// Drucker-Prager projection with hardening of the plastic amount q)
void return_map(const aep_params& P, int mat, V3& S, double& q) {
    if (mat == AEP_SNOW) {
        for (int a = 0; a < 3; ++a) S[a] = std::min(std::max(S[a], 1.0 - P.snow.theta_c), 1.0 + P.snow.theta_s);
        return;
    }
    double lambda, mu;
    lame(P.sand.E, P.sand.nu, lambda, mu);
    double phiF = (P.sand.h0 + (P.sand.h1 * q - P.sand.h3) * std::exp(-P.sand.h2 * q)) * kPi / 180.0;
    double alpha = std::sqrt(2.0 / 3.0) * 2.0 * std::sin(phiF) / (3.0 - std::sin(phiF));
    V3 ln{std::log(S[0]), std::log(S[1]), std::log(S[2])};
    double tr = ln[0] + ln[1] + ln[2];
    V3 dev{ln[0] - tr / 3.0, ln[1] - tr / 3.0, ln[2] - tr / 3.0};
    double nd = norm(dev);
    double dg = nd + (3.0 * lambda + 2.0 * mu) / 2.0 / mu * tr * alpha;
    if (dg <= 0.0) {
    } else if (nd == 0.0 || tr > 0.0) {
        S = V3{1, 1, 1};
        q += norm(ln);
    } else {
        for (int a = 0; a < 3; ++a) S[a] = std::exp(ln[a] - dg * dev[a] / nd);
        q += dg;
    }
}

// HybridSolver.cpp:553-609 + :612-723 for the particles; fused per particle
void plasticity_particles(Oracle& o, double dt) {
    const aep_params& P = o.prm;
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < o.np; ++p) {
        M3 G = grad_gather(o.W, p, o.gvbf);
        M3 F = o.Fe[p];
        M3 GF = mul(G, F);
        M3 Ftr = F;
        for (int k = 0; k < 9; ++k) Ftr[k] += dt * GF[k];
        M3 U, V;
        V3 S;
        svd3(Ftr, U, S, V);
        return_map(P, o.mat[p], S, o.plastic[p]);
        M3 Ds{}, Dinv{};
        for (int a = 0; a < 3; ++a) { E(Ds, a, a) = S[a]; E(Dinv, a, a) = 1.0 / S[a]; }
        M3 Ftot = mul(Ftr, o.Fp[p]);  // totalDeformationGradient, :618-619
        o.Fe[p] = mul(mul(U, Ds), transpose(V));
        o.Fp[p] = mul(mul(mul(V, Dinv), transpose(U)), Ftot);
    }
}

void mesh_g2p_and_plasticity(Oracle& o, double dt) {
    Mesh& me = o.mesh;
    // vertices: velocity, APIC with damp 1, advection (:748, :920-926, :948)
    std::vector<M3> Ge(me.nf);
    // element velocity gradients use the element weights at the old positions (:584-586)
#pragma omp parallel for schedule(static)
    for (int64_t f = 0; f < me.nf; ++f) Ge[f] = grad_gather(o.We, f, o.gvbf);
    // element APIC (:927-933) uses the old element positions and weights
    std::vector<V3> ve_unused(me.nf);
    g2p_set(o, o.We, me.xe, ve_unused, me.Be, 1.0, dt, false, false);
    g2p_set(o, o.Wv, me.xv, me.vv, me.Bv, 1.0, dt, true, true);
    // element velocity = mean of the vertex velocities (:749-756); element
    // positions = centroids of the new vertex positions (LagrangianMesh.cpp:371-380)
#pragma omp parallel for schedule(static)
    for (int64_t f = 0; f < me.nf; ++f) {
        const auto& fc = me.faces[f];
        for (int a = 0; a < 3; ++a) {
            me.ve[f][a] = (me.vv[fc[0]][a] + me.vv[fc[1]][a] + me.vv[fc[2]][a]) / 3.0;
            me.xe[f][a] = (me.xv[fc[0]][a] + me.xv[fc[1]][a] + me.xv[fc[2]][a]) / 3.0;
        }
        // :591-606
        V3 d1, d2, d3o{E(me.D[f], 0, 2), E(me.D[f], 1, 2), E(me.D[f], 2, 2)};
        for (int a = 0; a < 3; ++a) {
            d1[a] = me.xv[fc[1]][a] - me.xv[fc[0]][a];
            d2[a] = me.xv[fc[2]][a] - me.xv[fc[0]][a];
        }
        V3 Gd = matvec(Ge[f], d3o);
        M3 D;
        for (int a = 0; a < 3; ++a) {
            E(D, a, 0) = d1[a];
            E(D, a, 1) = d2[a];
            E(D, a, 2) = dt * Gd[a] + d3o[a];
        }
        // :686-720
        M3 Q, R;
        gram_schmidt(D, Q, R);
        if (E(R, 2, 2) > 1.0) {
            E(R, 2, 2) = 1.0;
            E(R, 0, 2) = E(R, 1, 2) = 0.0;
        } else {
            double nf_ = me.stiffness * (E(R, 2, 2) - 1.0) * (E(R, 2, 2) - 1.0);
            double sf = me.shear * std::sqrt(E(R, 0, 2) * E(R, 0, 2) + E(R, 1, 2) * E(R, 1, 2));
            if (sf > me.friction * nf_) {
                E(R, 0, 2) *= me.friction * nf_ / sf;
                E(R, 1, 2) *= me.friction * nf_ / sf;
            }
        }
        V3 rc{E(R, 0, 2), E(R, 1, 2), E(R, 2, 2)};
        V3 d3 = matvec(Q, rc);
        for (int a = 0; a < 3; ++a) E(D, a, 2) = d3[a];
        me.D[f] = D;
    }
}

void rebuild_weights(Oracle& o) {
    if (o.np) build_weights(o.g, o.x, o.W);
    if (o.has_mesh) {
        build_weights(o.g, o.mesh.xv, o.Wv);
        build_weights(o.g, o.mesh.xe, o.We);
    }
}

// The loop body of HybridSolver::solve (:869-989), stopping after `stage`.
// dt_force drives the force pass and the grid update (:873,877), dt the rest (:878-955).
void step(Oracle& o, double dt_force, double dt, int stage) {
    compute_forces(o, dt_force);
    if (stage == AEP_STAGE_FORCES) return;
    update_grid_velocities(o, dt_force);
    collision(o);
    if (stage == AEP_STAGE_GRID) return;
    if (o.np) {
        // :903 velocity, :910-917 APIC (damp 0), :944 advection
        g2p_set(o, o.W, o.x, o.v, o.B, o.prm.particle_damp, dt, true, true);
        // F update and return mapping use the weights of the old positions
        plasticity_particles(o, dt);
    }
    if (o.has_mesh) mesh_g2p_and_plasticity(o, dt);
    rebuild_weights(o);
    p2g(o, false);
    o.steps++;
}

// RegularGrid::max_velocity / CFL_condition (RegularGrid.cpp:188-200, RegularGrid.h:60)
double cfl_condition(const Oracle& o) {
    double vmax = 0.0;
    for (const V3& v : o.gv) vmax = std::max(vmax, norm(v));
    double hmin = std::min(o.g.h[0], std::min(o.g.h[1], o.g.h[2]));
    return vmax / hmin;
}

// HybridSolver::solve (:827-989) after the initial weights and P2G (orc_init with
// volumes): Dt from the P2G velocities; per iteration the force pass and grid
// update use the previous Dt, the new Dt (with the 1/60 s frame clamp) drives
// the rest.  Stops when t > maxt or after max_steps iterations (0: no limit).
// frame_t, if given, receives t after each completed frame (up to max_frames).
int64_t solve(Oracle& o, double cfl, double maxt, int64_t max_steps, double* t_out, int* frames_out,
              double* frame_t, int max_frames, double* dt_trace, int64_t trace_cap) {
    double t = 0.0, inner = 0.0;
    double Dt = cfl / std::max(3e2, cfl_condition(o));
    int frames = 0;
    int64_t it = 0;
    const double frame_dt = 1.0 / 60.0;
    while (t <= maxt && (max_steps <= 0 || it < max_steps)) {
        compute_forces(o, Dt);
        update_grid_velocities(o, Dt);
        Dt = cfl / std::max(3e2, cfl_condition(o));
        if (inner + Dt >= frame_dt) {
            Dt = frame_dt - inner;
            t += frame_dt;
            inner = 0.0;
            if (frame_t && frames < max_frames) frame_t[frames] = t;
            ++frames;
        } else {
            inner += Dt;
        }
        if (dt_trace && it < trace_cap) dt_trace[it] = Dt;
        collision(o);
        if (o.np) {
            g2p_set(o, o.W, o.x, o.v, o.B, o.prm.particle_damp, Dt, true, true);
            plasticity_particles(o, Dt);
        }
        if (o.has_mesh) mesh_g2p_and_plasticity(o, Dt);
        rebuild_weights(o);
        p2g(o, false);
        o.steps++;
        ++it;
    }
    if (t_out) *t_out = t;
    if (frames_out) *frames_out = frames;
    return it;
}

}  // namespace

// =========================== C API (ctypes) ===========================================
extern "C" {

void* orc_create(const aep_grid_desc* gd, const aep_params* prm) {
    Oracle* o = new Oracle();
    for (int a = 0; a < 3; ++a) {
        o->g.min[a] = gd->min[a];
        o->g.res[a] = gd->res[a];
        o->g.h[a] = (gd->max[a] - gd->min[a]) / gd->res[a];
    }
    o->prm = *prm;
    return o;
}

void orc_destroy(void* h) { delete (Oracle*)h; }

int orc_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

// same layouts as aep_set_particles
int orc_set_particles(void* h, int64_t n, const double* x, const double* v, const double* B,
                      const double* Fe, const double* Fp, const double* m, const double* vol,
                      const double* plastic, const uint8_t* mat) {
    Oracle* o = (Oracle*)h;
    o->np = n;
    o->x.resize(n); o->v.resize(n); o->B.resize(n); o->Fe.resize(n); o->Fp.resize(n);
    o->m.resize(n); o->vol.resize(n); o->rho.assign(n, 0.0); o->plastic.resize(n); o->mat.resize(n);
    for (int64_t p = 0; p < n; ++p) {
        for (int a = 0; a < 3; ++a) {
            o->x[p][a] = x[a * n + p];
            o->v[p][a] = v ? v[a * n + p] : 0.0;
            for (int b = 0; b < 3; ++b) E(o->B[p], a, b) = B ? B[a * 3 * n + b * n + p] : 0.0;
        }
        for (int k = 0; k < 9; ++k) {
            o->Fe[p][k] = Fe[9 * p + k];
            o->Fp[p][k] = Fp ? Fp[9 * p + k] : (k % 4 == 0 ? 1.0 : 0.0);
        }
        o->m[p] = m[p];
        o->vol[p] = vol ? vol[p] : 0.0;
        o->mat[p] = mat ? mat[p] : (uint8_t)AEP_SAND;
        o->plastic[p] = plastic ? plastic[p] : 0.0;
    }
    return 0;
}

// LagrangianMesh ctor arguments (LagrangianMesh.cpp:127-146).  d, drest: three
// Nf x 3 column-major blocks (directions 1 | 2 | 3).  faces: Nf x 3 column-major.
int orc_set_mesh(void* h, int64_t nv, int64_t nf, const double* xv, const int32_t* faces,
                 const double* vv, const double* ve, const double* mv, const double* volv,
                 const double* me_, const double* vole, const double* d, const double* drest,
                 double mu, double lambda, double shear, double stiffness, double friction) {
    Oracle* o = (Oracle*)h;
    Mesh& me = o->mesh;
    o->has_mesh = true;
    me.nv = nv; me.nf = nf;
    me.fixed.clear();
    me.xv.resize(nv); me.vv.resize(nv); me.Bv.assign(nv, M3{}); me.mv.resize(nv); me.volv.resize(nv);
    me.xe.resize(nf); me.ve.resize(nf); me.Be.assign(nf, M3{}); me.me.resize(nf); me.vole.resize(nf);
    me.faces.resize(nf); me.D.resize(nf); me.Drest.resize(nf);
    for (int64_t i = 0; i < nv; ++i) {
        for (int a = 0; a < 3; ++a) {
            me.xv[i][a] = xv[a * nv + i];
            me.vv[i][a] = vv ? vv[a * nv + i] : 0.0;
        }
        me.mv[i] = mv[i];
        me.volv[i] = volv ? volv[i] : 0.0;
    }
    for (int64_t f = 0; f < nf; ++f) {
        for (int c = 0; c < 3; ++c) me.faces[f][c] = faces[c * nf + f];
        for (int a = 0; a < 3; ++a) me.ve[f][a] = ve ? ve[a * nf + f] : 0.0;
        me.me[f] = me_[f];
        me.vole[f] = vole[f];
        for (int c = 0; c < 3; ++c)
            for (int a = 0; a < 3; ++a) {
                E(me.D[f], a, c) = d[c * 3 * nf + a * nf + f];
                E(me.Drest[f], a, c) = drest[c * 3 * nf + a * nf + f];
            }
        for (int a = 0; a < 3; ++a)  // updateElementPositions at construction (:187)
            me.xe[f][a] = (me.xv[me.faces[f][0]][a] + me.xv[me.faces[f][1]][a] + me.xv[me.faces[f][2]][a]) / 3.0;
    }
    me.mu = mu; me.lambda = lambda; me.shear = shear; me.stiffness = stiffness; me.friction = friction;
    return 0;
}

int orc_set_levelset(void* h, const aep_sdf* s, int32_t n) {
    Oracle* o = (Oracle*)h;
    o->shapes.clear();
    for (int i = 0; i < n; ++i) {
        Shape sh;
        sh.type = s[i].type;
        for (int k = 0; k < 6; ++k) sh.p[k] = s[i].p[k];
        o->shapes.push_back(sh);
    }
    return 0;
}

// weights + first P2G of solve (:829-855)
int orc_init(void* h, int compute_volumes) {
    Oracle* o = (Oracle*)h;
    rebuild_weights(*o);
    p2g(*o, compute_volumes != 0);
    return 0;
}

int64_t orc_solve(void* h, double cfl, double maxt, int64_t max_steps, double* t_out, int* frames_out,
                  double* frame_t, int max_frames, double* dt_trace, int64_t trace_cap) {
    return solve(*(Oracle*)h, cfl, maxt, max_steps, t_out, frames_out, frame_t, max_frames, dt_trace, trace_cap);
}

// vertex_is_fixed: nv doubles, nonzero = fixed (LagrangianMesh::bindConstraints); null clears
int orc_set_fixed_vertices(void* h, int64_t nv, const double* vertex_is_fixed) {
    Oracle* o = (Oracle*)h;
    if (!vertex_is_fixed) {
        o->mesh.fixed.clear();
        return 0;
    }
    if (!o->has_mesh || nv != o->mesh.nv) return 1;
    o->mesh.fixed.assign((size_t)nv, 0);
    for (int64_t v = 0; v < nv; ++v) o->mesh.fixed[v] = vertex_is_fixed[v] != 0.0;
    return 0;
}

int orc_step(void* h, double dt_force, double dt, int stage) {
    step(*(Oracle*)h, dt_force, dt, stage);
    return 0;
}

int orc_get_particles(void* h, int64_t n, double* x, double* v, double* B, double* Fe, double* Fp,
                      double* vol, double* plastic) {
    Oracle* o = (Oracle*)h;
    if (n != o->np) return 1;
    for (int64_t p = 0; p < n; ++p) {
        for (int a = 0; a < 3; ++a) {
            if (x) x[a * n + p] = o->x[p][a];
            if (v) v[a * n + p] = o->v[p][a];
            if (B)
                for (int b = 0; b < 3; ++b) B[a * 3 * n + b * n + p] = E(o->B[p], a, b);
        }
        for (int k = 0; k < 9; ++k) {
            if (Fe) Fe[9 * p + k] = o->Fe[p][k];
            if (Fp) Fp[9 * p + k] = o->Fp[p][k];
        }
        if (vol) vol[p] = o->vol[p];
        // sand: plasticAmount; snow: J_P = det F_P (the quantity the step reads)
        if (plastic) plastic[p] = o->mat[p] == AEP_SNOW ? det(o->Fp[p]) : o->plastic[p];
    }
    return 0;
}

int orc_get_mesh(void* h, double* xv, double* vv, double* Bv, double* xe, double* ve, double* Be,
                 double* d) {
    Oracle* o = (Oracle*)h;
    Mesh& me = o->mesh;
    int64_t nv = me.nv, nf = me.nf;
    for (int64_t i = 0; i < nv; ++i)
        for (int a = 0; a < 3; ++a) {
            if (xv) xv[a * nv + i] = me.xv[i][a];
            if (vv) vv[a * nv + i] = me.vv[i][a];
            if (Bv)
                for (int b = 0; b < 3; ++b) Bv[a * 3 * nv + b * nv + i] = E(me.Bv[i], a, b);
        }
    for (int64_t f = 0; f < nf; ++f) {
        for (int a = 0; a < 3; ++a) {
            if (xe) xe[a * nf + f] = me.xe[f][a];
            if (ve) ve[a * nf + f] = me.ve[f][a];
            if (Be)
                for (int b = 0; b < 3; ++b) Be[a * 3 * nf + b * nf + f] = E(me.Be[f], a, b);
        }
        if (d)
            for (int c = 0; c < 3; ++c)
                for (int a = 0; a < 3; ++a) d[c * 3 * nf + a * nf + f] = E(me.D[f], a, c);
    }
    return 0;
}

// dense grid in reference order: mass Ng, vel/vbf/force Ng x 3 column-major
int orc_get_grid(void* h, double* mass, double* vel, double* vbf, double* force) {
    Oracle* o = (Oracle*)h;
    int64_t ng = o->g.ng();
    for (int64_t n = 0; n < ng; ++n) {
        if (mass) mass[n] = o->gm.empty() ? 0.0 : o->gm[n];
        for (int a = 0; a < 3; ++a) {
            if (vel) vel[a * ng + n] = o->gv.empty() ? 0.0 : o->gv[n][a];
            if (vbf) vbf[a * ng + n] = o->gvbf.empty() ? 0.0 : o->gvbf[n][a];
            if (force) force[a * ng + n] = o->gf.empty() ? 0.0 : o->gf[n][a];
        }
    }
    return 0;
}

// the per-particle "cauchyStress" (incl. volume) of the last force pass, 9 per particle
int orc_get_stress(void* h, int64_t n, double* st) {
    Oracle* o = (Oracle*)h;
    if (n != o->np || (int64_t)o->last_stress.size() != n) return 1;
    for (int64_t p = 0; p < n; ++p)
        for (int k = 0; k < 9; ++k) st[9 * p + k] = o->last_stress[p][k];
    return 0;
}

// building blocks for known-answer tests
void orc_svd3(const double* A, double* U, double* s, double* V) {
    M3 a, u, v;
    V3 sv;
    for (int k = 0; k < 9; ++k) a[k] = A[k];
    svd3(a, u, sv, v);
    for (int k = 0; k < 9; ++k) { U[k] = u[k]; V[k] = v[k]; }
    for (int k = 0; k < 3; ++k) s[k] = sv[k];
}
// singular-value return map of one particle (mat: AEP_SNOW / AEP_SAND); s in/out, q in/out
void orc_return_map(const aep_params* prm, int mat, double* s, double* q) {
    V3 S{s[0], s[1], s[2]};
    return_map(*prm, mat, S, *q);
    for (int a = 0; a < 3; ++a) s[a] = S[a];
}
double orc_cubic(double x) { return cubic_B_spline(x); }
double orc_dcubic(double x) { return Dcubic_B_spline(x); }
void orc_gram_schmidt(const double* D, double* Q, double* R) {
    M3 d, q, r;
    for (int k = 0; k < 9; ++k) d[k] = D[k];
    gram_schmidt(d, q, r);
    for (int k = 0; k < 9; ++k) { Q[k] = q[k]; R[k] = r[k]; }
}
// weights of one particle: returns count, writes (node, w, g0, g1, g2)
int orc_particle_weights(void* h, const double* pos, int64_t* node, double* w, double* g) {
    Oracle* o = (Oracle*)h;
    int c = 0;
    particle_stencil(o->g, V3{pos[0], pos[1], pos[2]}, [&](int64_t n, double ww, double a, double b, double cc) {
        node[c] = n; w[c] = ww; g[3 * c] = a; g[3 * c + 1] = b; g[3 * c + 2] = cc; ++c;
    });
    return c;
}

}  // extern "C"
