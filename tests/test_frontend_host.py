"""Host-side behaviour of the Python front end (tileqr), no GPU needed: the
argument checks NextLA's helpers make before touching an array, the method
arities, one element type per call, and the refusal of host tensors (the
product path has no CPU fallback)."""
import pytest
import torch


@pytest.fixture(scope="module")
def tq():
    import tileqr
    return tileqr


def test_method_arities(tq):
    """Each method takes its NextLA argument list or the short helper form."""
    with pytest.raises(TypeError, match="no method with 3 arguments"):
        tq.geqr2(1, 2, 3)
    with pytest.raises(TypeError, match="no method with 4 arguments"):
        tq.geqrt(1, 2, 3, 4)
    with pytest.raises(TypeError, match="no method with 5 arguments"):
        tq.tsmqr(1, 2, 3, 4, 5)


def test_host_tensors_are_refused(tq):
    """Host arrays raise before any pointer is taken: there is no CPU path."""
    A = torch.zeros((8, 8), dtype=torch.float64).t()
    T = torch.zeros((4, 8), dtype=torch.float64).t().t()
    with pytest.raises(TypeError, match="CUDA tensors"):
        tq.geqrt(A, T)
    with pytest.raises(TypeError, match="CUDA tensors"):
        tq.geqr2(8, 8, A, torch.zeros(8, dtype=torch.float64), None)


def test_one_element_type_per_call(tq):
    f64 = torch.zeros(2, dtype=torch.float64)
    f32 = torch.zeros(2, dtype=torch.float32)
    assert tq._prefix(f64, None, f64) == "d"
    assert tq._prefix(f32) == "s"
    assert tq._prefix(torch.zeros(2, dtype=torch.complex128)) == "z"
    assert tq._prefix(torch.zeros(2, dtype=torch.complex64)) == "c"
    with pytest.raises(TypeError, match="one element type"):
        tq._prefix(f64, f32)
    with pytest.raises(TypeError, match="unsupported element type"):
        tq._prefix(torch.zeros(2, dtype=torch.int32))


def test_larft_tau_length_checks(tq):
    """larft!'s helper form checks length(tau) against V first
    (src/larft.jl:256-268)."""
    V = torch.zeros((6, 3), dtype=torch.float64)
    with pytest.raises(tq.ArgumentError, match="columnwise storage"):
        tq.larft("F", "C", V, torch.zeros(2, dtype=torch.float64), torch.zeros((3, 3), dtype=torch.float64))
    with pytest.raises(tq.ArgumentError, match="rowwise storage"):
        tq.larft("F", "R", V, torch.zeros(3, dtype=torch.float64), torch.zeros((6, 6), dtype=torch.float64))


def test_unmqr_helper_checks(tq):
    """unmqr!'s helper form: ib > 0, A's rows equal the order of Q, and A has
    at least k columns (src/unmqr.jl:196-222)."""
    C = torch.zeros((8, 5), dtype=torch.float64)
    with pytest.raises(tq.ArgumentError, match="Block size ib must be positive"):
        tq.unmqr("L", "N", torch.zeros((8, 4), dtype=torch.float64), torch.zeros((0, 4), dtype=torch.float64), C)
    with pytest.raises(tq.ArgumentError, match="rows must match"):
        tq.unmqr("L", "N", torch.zeros((7, 4), dtype=torch.float64), torch.zeros((2, 4), dtype=torch.float64), C)
    with pytest.raises(tq.ArgumentError, match="columns"):
        tq.unmqr("L", "N", torch.zeros((8, 2), dtype=torch.float64), torch.zeros((2, 4), dtype=torch.float64), C)


def test_argument_error_is_a_value_error(tq):
    """ArgumentError mirrors Julia's and is a ValueError for Python callers."""
    assert issubclass(tq.ArgumentError, ValueError)
