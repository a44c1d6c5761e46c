"""Direct parity of the mixed path's factorisation kernels with FP64 computations on
the same operands, through the kernel-check entry points of the C-ABI
(uchol_check_schur_update, uchol_check_diag_panel).

Tensor-core Schur update C -= W L^T (k_tc_gemm), one test per tile class: whole tiles
round robin, a launch split in K (stream-K, with its fixup), an update of a super-block's
own columns over a K range that starts inside the operands, a contribution block whose
last row tile is partial, and one CTA walking every tile.  Bound per entry:
c * u * sum_k |W_ik| |L_jk| with u = 2^-10 for TF32 operands (FP32 rounded inside the
MMA) and u = 2^-22 for BF16 (operands rounded to BF16 on the host, so only the FP32
accumulation differs from the FP64 product of the same values).

Outer block of the mixed path (k_diag_block + k_panel_solve): the staged W = L D
operands are rounded to TF32 to nearest.  D is FP64, computed from
the FP32 block with FP32 L, so recomputing D in FP64 from the kernel's own L
(d_r = a_rr - sum_k d_k L_rk^2) must give the same D to FP64 rounding; D, L against an
FP64 LDL^T of the block within FP32 accuracy times the block's growth; pivot counts as
the reference's rule gives them (UtduNumericFactorization.cs:553-592)."""
import ctypes as C

import numpy as np
import pytest

from magla_gb300 import _native
from magla_gb300.errors import raise_for_status

pytestmark = pytest.mark.gpu


def bf16_round(a):
    """Round FP32 to the nearest BF16 value (ties to even), as the staging copies do."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def schur_update(bf16, m, w, c0, cend, kbeg, kn, ld, max_ctas=0, seed=0):
    lib = _native.gpu()
    rng = np.random.default_rng(seed)
    front = np.asfortranarray(np.tril(rng.uniform(-1.0, 1.0, (m, m))).astype(np.float32))
    W = np.ascontiguousarray(rng.uniform(-1.0, 1.0, (m, ld)).astype(np.float32))
    L = np.ascontiguousarray(rng.uniform(-1.0, 1.0, (m, ld)).astype(np.float32))
    # K runs in whole 128-byte blocks: the operand columns past kbeg + kn are zero, as in the
    # factorisation's staging copies
    W[:, kbeg + kn:] = 0.0
    L[:, kbeg + kn:] = 0.0
    out = np.zeros((m, m), np.float32, order="F")
    tiles, split = C.c_int64(), C.c_int()
    st = lib.uchol_check_schur_update(int(bf16), m, w, c0, cend, kbeg, kn, front.ctypes.data, W.ctypes.data,
                                      L.ctypes.data, ld, max_ctas, out.ctypes.data, C.byref(tiles), C.byref(split))
    raise_for_status(st, lib.uchol_last_error())
    Wr, Lr = (bf16_round(W), bf16_round(L)) if bf16 else (W, L)
    Wk = Wr[:, kbeg:kbeg + kn].astype(np.float64)
    Lk = Lr[:, kbeg:kbeg + kn].astype(np.float64)
    ref = front.astype(np.float64)
    ref[:, c0:cend] -= Wk @ Lk[c0:cend].T
    scale = np.abs(Wk) @ np.abs(Lk[c0:cend]).T
    return front, out, ref, scale, tiles.value, split.value


def check_update(front, out, ref, scale, c0, cend, u):
    m = front.shape[0]
    lower = np.tril(np.ones((m, m), bool))
    cols = np.zeros(m, bool)
    cols[c0:cend] = True
    region = (lower & cols[None, :])[:, c0:cend]
    err = np.abs(out.astype(np.float64) - ref)[:, c0:cend]
    bound = 4.0 * u * scale + 2.0 ** -23 * np.abs(ref[:, c0:cend])
    assert np.all(err[region] <= bound[region]), f"max error / bound {np.max((err / bound)[region]):.3f}"
    # columns outside the job are untouched (bit for bit)
    assert np.array_equal(out[:, ~cols], front[:, ~cols])


TF32_U, BF16_U = 2.0 ** -10, 2.0 ** -22


@pytest.mark.parametrize("bf16", [0, 1])
def test_whole_tiles_round_robin(gpu_lib, bf16):
    m, w = 4300, 300
    front, out, ref, scale, tiles, split = schur_update(bf16, m, w, w, m, 0, w, 320)
    assert tiles > 152 and split == 0
    check_update(front, out, ref, scale, w, m, BF16_U if bf16 else TF32_U)


@pytest.mark.parametrize("bf16", [0, 1])
def test_stream_k_split_tile(gpu_lib, bf16):
    # one tile, K = 2048 -> split over several CTAs, partial tiles added in CTA order
    m, w = 2088, 2048
    front, out, ref, scale, tiles, split = schur_update(bf16, m, w, w, m, 0, w, 2048, seed=1)
    assert tiles == 1 and split == 1
    check_update(front, out, ref, scale, w, m, BF16_U if bf16 else TF32_U)


def test_split_is_deterministic(gpu_lib):
    a = schur_update(0, 2088, 2048, 2048, 2088, 0, 2048, 2048, seed=1)[1]
    b = schur_update(0, 2088, 2048, 2048, 2088, 0, 2048, 2048, seed=1)[1]
    assert np.array_equal(a, b)


@pytest.mark.parametrize("bf16", [0, 1])
def test_super_block_k_range_own_columns(gpu_lib, bf16):
    # columns [512, 640) of the panel take the super-block's own earlier columns [384, 512)
    m, w = 900, 700
    front, out, ref, scale, tiles, split = schur_update(bf16, m, w, 512, 640, 384, 128, 704, seed=2)
    assert split == 0
    check_update(front, out, ref, scale, 512, 640, BF16_U if bf16 else TF32_U)


def test_super_block_update_split_in_k(gpu_lib):
    # columns [1024, 1152) of the panel take every earlier column of the supernode (K = 1024)
    m, w = 1600, 1400
    front, out, ref, scale, tiles, split = schur_update(0, m, w, 1024, 1152, 0, 1024, 1408, seed=3)
    assert tiles < 152 and split == 1
    check_update(front, out, ref, scale, 1024, 1152, TF32_U)


@pytest.mark.parametrize("bf16", [0, 1])
def test_contribution_with_partial_last_row_tile(gpu_lib, bf16):
    m, w = 1000, 137   # 863 trailing rows: 3 full row tiles of 256 and one of 95
    front, out, ref, scale, tiles, split = schur_update(bf16, m, w, w, m, 0, w, 192, seed=4)
    check_update(front, out, ref, scale, w, m, BF16_U if bf16 else TF32_U)


def test_one_cta_walks_every_tile(gpu_lib):
    m, w = 1300, 260
    front, out, ref, scale, tiles, split = schur_update(0, m, w, w, m, 0, w, 320, max_ctas=1, seed=5)
    assert tiles > 10 and split == 0
    check_update(front, out, ref, scale, w, m, TF32_U)


# ---- outer block: k_diag_block + k_panel_solve ----------------------------------

def diag_panel(front, threshold=1e-13, regularization=1e-10, allow=1):
    lib = _native.gpu()
    m, nb = front.shape
    A = np.asfortranarray(front.astype(np.float32))
    Lo = np.zeros((m, nb), np.float32, order="F")
    D = np.zeros(nb)
    Ws = np.zeros((m, nb), np.float32, order="F")
    counts = (C.c_int * 3)()
    st = lib.uchol_check_diag_panel(m, nb, A.ctypes.data, threshold, regularization, allow, Lo.ctypes.data,
                                    D.ctypes.data, Ws.ctypes.data, counts)
    raise_for_status(st, lib.uchol_last_error())
    return A, Lo, D, Ws, list(counts)


def ldlt64(A11):
    n = A11.shape[0]
    L = np.eye(n)
    D = np.zeros(n)
    S = A11.astype(np.float64).copy()
    for k in range(n):
        D[k] = S[k, k]
        L[k + 1:, k] = S[k + 1:, k] / D[k]
        S[k + 1:, k + 1:] -= np.outer(L[k + 1:, k], L[k + 1:, k]) * D[k]
    return L, D


def spd_front(m, nb, seed):
    rng = np.random.default_rng(seed)
    G = rng.standard_normal((m, m + 20))
    A = G @ G.T / (m + 20) + 0.5 * np.eye(m)
    return A[:, :nb]


@pytest.mark.parametrize("m,nb", [(128, 128), (300, 128), (517, 96), (64, 33)])
def test_outer_block_matches_fp64_ldlt(gpu_lib, m, nb):
    A, Lg, Dg, Ws, counts = diag_panel(spd_front(m, nb, seed=m + nb))
    assert counts == [0, 0, -1]
    A64 = A.astype(np.float64)
    Lr, Dr = ldlt64(A64[:nb])
    L21r = np.linalg.solve(Lr, A64[nb:].T).T / Dr   # A21 L11^-T D^-1
    assert np.max(np.abs(Dg - Dr) / np.abs(Dr)) < 1e-4
    # the kernel writes the lower triangle of L11 (its upper part keeps A)
    assert np.max(np.abs(np.tril(Lg[:nb].astype(np.float64)) - np.tril(Lr))) < 1e-4
    if m > nb:
        assert np.max(np.abs(Lg[nb:] - L21r)) < 1e-4 * max(1.0, np.max(np.abs(L21r)))
        # the staged W = L D rows of the panel solve, rounded to TF32 (10 mantissa bits, nearest)
        W = Lg[nb:].astype(np.float64) * Dg
        assert np.all(np.abs(Ws[nb:] - W) <= 2.0 ** -11 * np.abs(W) * (1 + 1e-3) + 1e-30)


@pytest.mark.parametrize("m,nb", [(128, 128), (517, 96)])
def test_pivots_are_fp64_of_the_kernels_own_l(gpu_lib, m, nb):
    """D recomputed in FP64 from the FP32 block and the kernel's FP32 L, in the kernel's order."""
    A, Lg, Dg, _, _ = diag_panel(spd_front(m, nb, seed=7))
    L = Lg[:nb].astype(np.float64)
    for r in range(nb):
        d = float(A[r, r])
        for k in range(r):
            d -= Dg[k] * (L[r, k] * L[r, k])
        assert abs(d - Dg[r]) <= 1e-13 * abs(Dg[r]), r


def test_pivot_rule_counts_regularised_and_negative(gpu_lib):
    nb = 40
    A = np.zeros((nb, nb))
    d = np.linspace(1.0, 2.0, nb)
    d[5] = 1e-20      # below tol * scale: regularised
    d[17] = -3.0      # negative: regularised and counted negative
    d[33] = 0.0
    A[np.arange(nb), np.arange(nb)] = d
    A[20, 19] = 0.25   # a coupling inside the block
    scale = np.max(np.abs(d))
    A2, Lg, Dg, _, counts = diag_panel(A, threshold=1e-13 * scale, regularization=1e-10 * scale, allow=1)
    assert counts == [3, 1, -1]
    assert Dg[5] == Dg[17] == Dg[33] == 1e-10 * scale
    _, _, _, _, strict = diag_panel(A, threshold=1e-13 * scale, regularization=1e-10 * scale, allow=0)
    assert strict[2] == 5   # the first rejected column
