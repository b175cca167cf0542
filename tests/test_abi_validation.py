"""Argument checks of the C ABI, called through the library itself without a GPU: null handles,
bad sizes and bad scalars return their status codes before any CUDA call, and destroying a
null handle is a no-op.  Where a check needs non-null pointers, the call passes a fake
address only when an earlier check of the same call fails first, so nothing is dereferenced
and no CUDA call is reached."""
import ctypes

import pytest

SC_OK, SC_BAD_ARG, SC_CAPACITY = 0, 1, 4
FAKE = ctypes.c_void_p(4096)  # never dereferenced: see the module docstring


@pytest.fixture(scope="module")
def lib():
    from scatter_gb300 import _native

    return _native.load()


def test_null_handles(lib):
    for fn in ("sc_newmark_run", "sc_nb_run", "sc_batch_run"):
        assert getattr(lib, fn)(None, 0, 1) == SC_BAD_ARG, fn
    assert lib.sc_newmark_set_predictor(None, 0) == SC_BAD_ARG
    assert lib.sc_nb_set_predictor(None, 2) == SC_BAD_ARG
    for fn in ("sc_newmark_destroy", "sc_nb_destroy", "sc_batch_destroy"):
        assert getattr(lib, fn)(None) == SC_OK, fn


def test_newmark_create_checks(lib):
    h = ctypes.c_void_p()
    n = 10
    ws_need = lib.sc_newmark_workspace_doubles(n, 0)
    def create(out, n_eq, dt, rtol, max_iter, ws, ws_doubles):
        # rowptr cols M C K A, the scalars, then u v a, the workspace and the stream
        return lib.sc_newmark_create(out, n_eq, *[FAKE] * 6, dt, rtol, max_iter, FAKE, FAKE, FAKE, ws, ws_doubles,
                                     None)

    assert create(None, n, 1e-3, 1e-12, 10, FAKE, ws_need) == SC_BAD_ARG  # no handle slot
    assert create(ctypes.byref(h), 0, 1e-3, 1e-12, 10, FAKE, ws_need) == SC_BAD_ARG  # no equations
    assert create(ctypes.byref(h), n, 0.0, 1e-12, 10, FAKE, ws_need) == SC_BAD_ARG  # dt
    assert create(ctypes.byref(h), n, 1e-3, 0.0, 10, FAKE, ws_need) == SC_BAD_ARG  # tolerance
    assert create(ctypes.byref(h), n, 1e-3, 1e-12, 0, FAKE, ws_need) == SC_BAD_ARG  # iteration cap
    assert create(ctypes.byref(h), n, 1e-3, 1e-12, 10, FAKE, ws_need - 1) == SC_BAD_ARG  # workspace size
    assert create(ctypes.byref(h), n, 1e-3, 1e-12, 10, ctypes.c_void_p(4104), ws_need) == SC_BAD_ARG  # alignment
    assert h.value is None
    # per equation: 9 solver vectors and the warm start's 8 history vectors
    assert lib.sc_newmark_workspace_doubles(2 * n, 0) - ws_need >= 17 * n


def test_predictor_order_range(lib):
    for order in (-1, 9):
        assert lib.sc_newmark_set_predictor(FAKE, order) == SC_BAD_ARG
        assert lib.sc_nb_set_predictor(FAKE, order) == SC_BAD_ARG


def test_size_checks(lib):
    assert lib.sc_batch_create(None, None, None, None, None) == SC_BAD_ARG
    assert lib.sc_rf_modes(1, 0, 8, 1.0, 1.0, 1.0, FAKE, None) == SC_BAD_ARG
    assert lib.sc_rf_modes(1, 4, 8, 1.0, 0.0, 1.0, FAKE, None) == SC_BAD_ARG
    assert lib.sc_rf_lognormal(0, FAKE, 4, 8, FAKE, 0.0, 1.0, FAKE, None) == SC_BAD_ARG
    # covariance model codes 0..2 only; the Matern model needs 0 < nu
    assert lib.sc_rf_modes_model(1, 4, 8, 3, 1.0, 1.0, 1.0, 1.0, None, FAKE, None) == SC_BAD_ARG
    assert lib.sc_rf_modes_model(1, 4, 8, 2, 0.0, 1.0, 1.0, 1.0, None, FAKE, None) == SC_BAD_ARG
    assert lib.sc_rf_modes_model(1, 4, 8, 1, 1.0, 1.0, -1.0, 1.0, None, FAKE, None) == SC_BAD_ARG
    assert lib.sc_element_matrices(0, 2, 5, None, None, None, None, None, None, None) == SC_BAD_ARG
    assert lib.sc_element_matrices(0, 2, -1, None, None, None, None, None, None, None) == SC_BAD_ARG
    assert lib.sc_combine(-1, 1.0, None, 1.0, None, 1.0, None, FAKE, None) == SC_BAD_ARG
    assert lib.sc_csr_row_sums(-1, None, None, 0, None, None) == SC_BAD_ARG
    assert lib.sc_csr_row_sums(5, None, FAKE, 0, FAKE, None) == SC_BAD_ARG


def test_noalloc_scan_limits(lib):
    assert lib.sc_exclusive_scan_i64_noalloc(-1, FAKE, FAKE, None) == SC_BAD_ARG
    assert lib.sc_exclusive_scan_i64_noalloc(4, None, FAKE, None) == SC_BAD_ARG
    assert lib.sc_exclusive_scan_i64_noalloc(8388608 + 1, FAKE, FAKE, None) == SC_CAPACITY
    assert b"exceeds the maximum" in lib.sc_last_error()


def test_status_strings_are_distinct(lib):
    texts = [lib.sc_status_string(c) for c in range(6)]
    assert len(set(texts)) == 6 and all(texts)
    assert lib.sc_status_string(99) == b"unknown status"


def test_node_block_option_and_residual_checks(lib):
    assert lib.sc_nb_set_options(None, 0) == SC_BAD_ARG
    flag = ctypes.c_int()
    assert lib.sc_nb_residual_fp64(None, ctypes.byref(flag)) == SC_BAD_ARG
    n = ctypes.c_int64()
    assert lib.sc_nb_a32_status(None, ctypes.byref(n), ctypes.byref(n), ctypes.byref(n), None) == SC_BAD_ARG
    ms = ctypes.c_float()
    assert lib.sc_nb_time_spmv_a32(None, 1, 5, ctypes.byref(ms), None) == SC_BAD_ARG
    order = ctypes.c_int()
    assert lib.sc_nb_warm_start_status(None, ctypes.byref(order), ctypes.byref(n)) == SC_BAD_ARG
    assert lib.sc_nb_status_to(None, FAKE) == SC_BAD_ARG
    assert lib.sc_newmark_status_to(None, FAKE) == SC_BAD_ARG


def test_batched_shape_checks(lib):
    assert lib.sc_batch_set_node_shape(None, 4, 256) == SC_BAD_ARG
    assert lib.sc_batch_set_node_shape_budget(None, 4, 256, 1) == SC_BAD_ARG


def test_csr_option_checks(lib):
    assert lib.sc_newmark_set_options(None, 0) == SC_BAD_ARG
    order, n = ctypes.c_int(), ctypes.c_int64()
    assert lib.sc_newmark_warm_start_status(None, ctypes.byref(order), ctypes.byref(n)) == SC_BAD_ARG
