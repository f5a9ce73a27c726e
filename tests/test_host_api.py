"""Host-side argument checks of the Python mirror of the reference API
(glagpu): the errors it raises before any device work, so these run without
a GPU. The reference raises DimensionMismatch for non-square input
(src/eigenSelfAdjoint.jl:230-243) and for mismatched EigenQ operands
(:25-27, :64-66)."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def G():
    import glagpu
    return glagpu


def test_symtridiagonal_lengths(G):
    G.SymTridiagonal(np.zeros(3), np.zeros(2))
    G.SymTridiagonal(np.zeros(0), np.zeros(0))
    with pytest.raises(G.DimensionMismatch):
        G.SymTridiagonal(np.zeros(3), np.zeros(3))


def test_quaternion_matrix_shape(G):
    G.QuaternionMatrix(np.zeros((3, 3, 4)))
    for bad in ((3, 3, 3), (3, 4, 4), (3, 3), (2, 3, 3, 4)):
        with pytest.raises(G.DimensionMismatch):
            G.QuaternionMatrix(np.zeros(bad))


def test_eigenq_uplo(G):
    with pytest.raises(ValueError):
        G.EigenQ(np.eye(3), np.zeros(2), uplo="X")
    q = G.EigenQ(np.eye(3), np.zeros(2), uplo="U")
    assert q.uplo == "U" and q.n == 3


def test_subsets_need_a_symtridiagonal(G):
    with pytest.raises(ValueError):
        G.eigvals(np.eye(3), irange=(1, 2))


def test_precision_limits_of_non_real_input(G):
    with pytest.raises(ValueError):
        G.eigen(np.eye(2, dtype=complex), precision="f32")
    with pytest.raises(ValueError):
        G.eigvals(G.QuaternionMatrix(np.zeros((2, 2, 4))), tol=1e-3)


def test_eigenq_operand_shapes(G):
    # lmul! needs size(Q, 1) rows, rmul! size(Q, 1) columns; checked before any device work
    q = G.EigenQ(np.eye(4), np.zeros(3))
    with pytest.raises(G.DimensionMismatch):
        q.lmul(np.zeros((3, 2)))
    with pytest.raises(G.DimensionMismatch):
        q.rmul(np.zeros((2, 3)))
    with pytest.raises(G.DimensionMismatch):
        q.lmul(np.zeros(4))
