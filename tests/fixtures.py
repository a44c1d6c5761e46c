"""Matrices of the reference's UCHOL test-suite (Tests/UCHOL/SymmetricUtduSolverTests.cs),
rebuilt with this project's seeded generator where the reference uses System.Random."""
import numpy as np

from magla_gb300 import SymmetricCSRMatrixBuilder
from magla_gb300 import generators as G


def diagonal(values):
    b = SymmetricCSRMatrixBuilder(len(values))
    for i, v in enumerate(values):
        b.AddToElement(i, i, v)
    return b.Build()


def tridiagonal(n, diag=4.0, off=-1.0):
    b = SymmetricCSRMatrixBuilder(n)
    for i in range(n):
        b.AddToElement(i, i, diag)
    for i in range(n - 1):
        b.AddToElement(i, i + 1, off)
    return b.Build()


def star(n=300):
    """One dense row (SymmetricUtduSolverTests.cs:351-357): exercises the dense-row branch of AMD."""
    b = SymmetricCSRMatrixBuilder(n)
    for i in range(1, n):
        b.AddToElement(0, i, -1.0)
    b.AddToElement(0, 0, n + 1.0)
    for i in range(1, n):
        b.AddToElement(i, i, 2.0)
    return b.Build()


def two_chains():
    b = SymmetricCSRMatrixBuilder(200)
    for i in range(99):
        b.AddToElement(i, i + 1, -1.0)
    for i in range(100, 199):
        b.AddToElement(i, i + 1, -1.0)
    for i in range(200):
        b.AddToElement(i, i, 4.0)
    return b.Build()


def random_matrix(n, density, seed):
    return G.random_spd(n, density, np.random.default_rng(seed))


def singular():
    b = SymmetricCSRMatrixBuilder(4)
    b.AddToElement(0, 0, 1.0)
    b.AddToElement(1, 1, 1.0)
    b.AddToElement(0, 1, 1.0)
    b.AddToElement(2, 2, 2.0)
    b.AddToElement(3, 3, 3.0)
    return b.Build()


def indefinite():
    b = SymmetricCSRMatrixBuilder(3)
    b.AddToElement(0, 0, 1.0)
    b.AddToElement(1, 1, 1.0)
    b.AddToElement(2, 2, 1.0)
    b.AddToElement(0, 1, 3.0)
    return b.Build()


# The 8x8 SPD system of the reference's workbook fixture (Tests/BiCGSTAB/CgComparisonData.cs:8-46),
# with its exact solution and its unpivoted L and U = D L^T factors.
CG_MATRIX = np.array([
    [741.7582417582419, 0, 0, 0, 0, 0, 0, 0],
    [0, 741.7582417582419, 0, 0, 0, 0, 0, 0],
    [0, 0, 741.7582417582419, 0, -192.30769230769232, -192.30769230769232, 0, 357.14285714285717],
    [0, 0, 0, 741.7582417582419, 0, 0, 0, 0],
    [0, 0, -192.30769230769232, 0, 741.7582417582419, 357.14285714285717, -549.4505494505495, -192.30769230769232],
    [0, 0, -192.30769230769232, 0, 357.14285714285717, 741.7582417582419, -164.83516483516485, -192.30769230769232],
    [0, 0, 0, 0, -549.4505494505495, -164.83516483516485, 741.7582417582419, 0],
    [0, 0, 357.14285714285717, 0, -192.30769230769232, -192.30769230769232, 0, 741.7582417582419],
])
CG_RHS = np.array([0.0, 0.0, 0.0, 0.0, 200.0, 0.0, 0.0, -1000.0])
CG_EXACT = np.array([0.0, 0.0, 0.8379999999999997, 0.0, 0.31800000000000006, -0.358, 0.15600000000000014,
                     -1.7619999999999996])
CG_LOWER = np.array([
    [1, 0, 0, 0, 0, 0, 0, 0],
    [0, 1, 0, 0, 0, 0, 0, 0],
    [0, 0, 1, 0, 0, 0, 0, 0],
    [0, 0, 0, 1, 0, 0, 0, 0],
    [0, 0, -0.25925925925925924, 0, 1, 0, 0, 0],
    [0, 0, -0.25925925925925924, 0, 0.4441176470588235, 1, 0, 0],
    [0, 0, 0, 0, -0.7941176470588235, 0.1425661914460285, 1, 0],
    [0, 0, 0.48148148148148145, 0, -0.14411764705882352, -0.09979633401221995, 0, 1],
])
CG_UPPER_DIAG = np.array([741.7582417582419, 741.7582417582419, 741.7582417582419, 741.7582417582419,
                          691.900691900692, 555.4298642533938, 294.1406861977128, 549.89816700611])


def cg_matrix():
    b = SymmetricCSRMatrixBuilder(8)
    for i in range(8):
        for j in range(i, 8):
            if CG_MATRIX[i, j] != 0.0:
                b.AddToElement(i, j, CG_MATRIX[i, j])
    return b.Build()
