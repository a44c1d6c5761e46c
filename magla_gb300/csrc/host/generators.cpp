// Seeded synthetic matrices used by the tests and the benchmark.  Every
// generator emits coordinate triplets in a fixed order and goes through
// csr_from_triplets, so the reference's construction rules (normalisation,
// ordered duplicate summation, the 1e-15 drop) apply exactly as they would
// for a matrix assembled with SymmetricCSRMatrixBuilder.
#include <array>
#include <cmath>

#include "generators.hpp"

namespace uchol {

namespace {
struct Triplets {
    std::vector<int> r, c;
    std::vector<double> v;
    void add(int i, int j, double x) {
        r.push_back(i);
        c.push_back(j);
        v.push_back(x);
    }
    UpperCsr build(int n) const {
        return csr_from_triplets(n, static_cast<int64_t>(r.size()), r.data(), c.data(), v.data());
    }
};
}  // namespace

// Same structure and values as the reference's FEM-like grid matrix
// (CAESolvers/UCHOL/UtduSolverBenchmark.cs:220-261 and
// Tests/UCHOL/SymmetricUtduSolverTests.cs:61-102): dof x dof coupling
// blocks between 6-neighbour nodes, diagonally dominant.
UpperCsr grid_matrix(int nx, int ny, int nz, int dof) {
    const int nodes = nx * ny * nz;
    Triplets t;
    std::vector<int> neighbours(nodes, 0);
    auto index = [&](int x, int y, int z) { return (z * ny + y) * nx + x; };
    auto couple = [&](int a, int b) {
        for (int d = 0; d < dof; ++d)
            for (int e = 0; e < dof; ++e) t.add(a * dof + d, b * dof + e, d == e ? -1.0 : -0.0625);
        neighbours[a]++;
        neighbours[b]++;
    };
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                int node = index(x, y, z);
                if (x + 1 < nx) couple(node, index(x + 1, y, z));
                if (y + 1 < ny) couple(node, index(x, y + 1, z));
                if (z + 1 < nz) couple(node, index(x, y, z + 1));
            }
    for (int node = 0; node < nodes; ++node)
        for (int d = 0; d < dof; ++d) {
            for (int e = d + 1; e < dof; ++e) t.add(node * dof + d, node * dof + e, -0.25);
            t.add(node * dof + d, node * dof + d, neighbours[node] * dof + 0.25 * (dof - 1) + 1.0);
        }
    return t.build(nodes * dof);
}

// 3D 7-point Laplacian on the interior nodes of an (nx+1)x(ny+1)x(nz+1)
// box with Dirichlet boundaries eliminated: 6 on the diagonal, -1 to each
// interior neighbour.
UpperCsr laplacian3d(int nx, int ny, int nz) {
    Triplets t;
    auto index = [&](int x, int y, int z) { return (z * ny + y) * nx + x; };
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                int i = index(x, y, z);
                t.add(i, i, 6.0);
                if (x + 1 < nx) t.add(i, index(x + 1, y, z), -1.0);
                if (y + 1 < ny) t.add(i, index(x, y + 1, z), -1.0);
                if (z + 1 < nz) t.add(i, index(x, y, z + 1), -1.0);
            }
    return t.build(nx * ny * nz);
}

// 2D Laplacian on an n x n interior grid, 5-point (4 on the diagonal) or
// 9-point (8 on the diagonal, -1 to all eight neighbours), plus a diagonal
// shift per node.
UpperCsr laplacian2d(int n, int stencil, const double* shift) {
    Triplets t;
    auto index = [&](int x, int y) { return y * n + x; };
    const double centre = stencil == 9 ? 8.0 : 4.0;
    for (int y = 0; y < n; ++y)
        for (int x = 0; x < n; ++x) {
            int i = index(x, y);
            t.add(i, i, centre + (shift ? shift[i] : 0.0));
            if (x + 1 < n) t.add(i, index(x + 1, y), -1.0);
            if (y + 1 < n) t.add(i, index(x, y + 1), -1.0);
            if (stencil == 9 && y + 1 < n) {
                if (x + 1 < n) t.add(i, index(x + 1, y + 1), -1.0);
                if (x > 0) t.add(i, index(x - 1, y + 1), -1.0);
            }
        }
    return t.build(n * n);
}

// Trilinear (Q1) hexahedron stiffness of a unit cube for E = 1, Poisson
// ratio nu, 2x2x2 Gauss quadrature; 24 x 24, dof order (node, xyz).
static std::array<double, 24 * 24> unit_hex_stiffness(double nu) {
    const double lam = nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
    const double mu = 1.0 / (2.0 * (1.0 + nu));
    const double g = 1.0 / std::sqrt(3.0);
    const int sx[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
    const int sy[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
    const int sz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
    std::array<double, 24 * 24> K{};
    for (int q = 0; q < 8; ++q) {
        double xi = sx[q] * g, eta = sy[q] * g, zeta = sz[q] * g;
        // Reference cube [-1,1]^3 mapped to the unit cube: dx = 0.5 dxi,
        // detJ = 1/8, weights 1.
        double dN[8][3];
        for (int a = 0; a < 8; ++a) {
            dN[a][0] = 0.125 * sx[a] * (1 + sy[a] * eta) * (1 + sz[a] * zeta) * 2.0;
            dN[a][1] = 0.125 * sy[a] * (1 + sx[a] * xi) * (1 + sz[a] * zeta) * 2.0;
            dN[a][2] = 0.125 * sz[a] * (1 + sx[a] * xi) * (1 + sy[a] * eta) * 2.0;
        }
        const double detJ = 0.125;
        for (int a = 0; a < 8; ++a)
            for (int b = 0; b < 8; ++b)
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) {
                        // K_ai,bj = lam dNa_i dNb_j + mu (dNa_j dNb_i + delta_ij dNa.dNb)
                        double v = lam * dN[a][i] * dN[b][j] + mu * dN[a][j] * dN[b][i];
                        if (i == j) v += mu * (dN[a][0] * dN[b][0] + dN[a][1] * dN[b][1] + dN[a][2] * dN[b][2]);
                        K[(3 * a + i) * 24 + 3 * b + j] += v * detJ;
                    }
    }
    return K;
}

ElasticityProblem elasticity_q1(int ex, int ey, int ez, const double* youngs, double nu, bool clamp_bottom) {
    const int nx = ex + 1, ny = ey + 1, nz = ez + 1;
    const int nodes = nx * ny * nz;
    const int n = 3 * nodes;
    auto node = [&](int x, int y, int z) { return (z * ny + y) * nx + x; };
    const auto K = unit_hex_stiffness(nu);
    const int ox[8] = {0, 1, 1, 0, 0, 1, 1, 0};
    const int oy[8] = {0, 0, 1, 1, 0, 0, 1, 1};
    const int oz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
    ElasticityProblem P;
    P.body_load.assign(n, 0.0);
    Triplets t;
    t.r.reserve(static_cast<size_t>(ex) * ey * ez * 300);
    t.c.reserve(t.r.capacity());
    t.v.reserve(t.r.capacity());
    int e = 0;
    for (int z = 0; z < ez; ++z)
        for (int y = 0; y < ey; ++y)
            for (int x = 0; x < ex; ++x, ++e) {
                const double E = youngs ? youngs[e] : 1.0;
                int dof[24];
                for (int a = 0; a < 8; ++a)
                    for (int i = 0; i < 3; ++i) dof[3 * a + i] = 3 * node(x + ox[a], y + oy[a], z + oz[a]) + i;
                // Each unordered pair is added once (upper triangle of the
                // element matrix), as a FEM code using the symmetric builder does.
                for (int p = 0; p < 24; ++p)
                    for (int q = p; q < 24; ++q) t.add(dof[p], dof[q], E * K[p * 24 + q]);
                for (int a = 0; a < 8; ++a) P.body_load[dof[3 * a + 2]] -= 0.125;  // unit body force in -z
            }
    P.matrix = t.build(n);
    if (clamp_bottom) {
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x)
                for (int i = 0; i < 3; ++i) P.clamped.push_back(3 * node(x, y, 0) + i);
        line_cross_zero(P.matrix, P.clamped);
    }
    return P;
}

// Dirichlet condition x[idx] = 0 applied with the reference's LineCross
// semantics (CAESolvers/SymmetricCSRMatrix.cs:125-167): couplings become
// explicit zeros, the diagonal becomes 1, the structure is unchanged.  With
// a zero prescribed value the right-hand side only needs rhs[idx] = 0,
// which callers apply.
void line_cross_zero(UpperCsr& m, const std::vector<int>& indices) {
    std::vector<char> fixed(m.n, 0);
    for (int idx : indices) {
        if (idx < 0 || idx >= m.n) throw std::out_of_range("constrained index out of range");
        if (m.diag_index[idx] < 0) throw std::runtime_error("diagonal position is absent from the sparse structure");
        fixed[idx] = 1;
    }
    for (int r = 0; r < m.n; ++r)
        for (int k = m.row_ptr[r]; k < m.row_ptr[r + 1]; ++k) {
            int c = m.col[k];
            if (c == r) continue;
            if (fixed[r] || fixed[c]) m.val[k] = 0.0;
        }
    for (int idx : indices) m.val[m.diag_index[idx]] = 1.0;
}

}  // namespace uchol
