// Synthetic test and benchmark matrices (host).
#pragma once

#include "symbolic.hpp"

namespace uchol {

UpperCsr grid_matrix(int nx, int ny, int nz, int dof);
UpperCsr laplacian3d(int nx, int ny, int nz);
UpperCsr laplacian2d(int n, int stencil, const double* shift);

struct ElasticityProblem {
    UpperCsr matrix;
    std::vector<double> body_load;  // consistent nodal load of a unit body force in -z
    std::vector<int> clamped;       // constrained equations (face z = 0)
};
// Q1 hexahedral linear elasticity on ex x ey x ez unit cubes; youngs holds
// one modulus per element (element order x fastest, then y, then z) or is
// null for E = 1.
ElasticityProblem elasticity_q1(int ex, int ey, int ez, const double* youngs, double nu, bool clamp_bottom);

void line_cross_zero(UpperCsr& m, const std::vector<int>& indices);

}  // namespace uchol
