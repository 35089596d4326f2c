"""The serving loop's host-side bounded wait (mcx_poll_flag), without a GPU: it returns
MCX_ERR_TIMEOUT when the flag stays below the target for the poll limit, and MCX_OK as soon
as another thread (standing in for the device) raises it."""
import ctypes as C
import threading
import time

import numpy as np
import pytest


def test_poll_flag_cap_runs_out_and_succeeds(mcxlib):
    from mcx import _lib as L
    lib = L.load()
    flag = np.zeros(1, np.uint32)
    ptr = flag.ctypes.data
    t0 = time.perf_counter()
    assert lib.mcx_poll_flag(ptr, 1, 2000, 1000) == L.MCX_ERR_TIMEOUT  # nothing sets it: the cap runs out
    assert time.perf_counter() - t0 < 5.0
    assert b"stayed below" in L.load().mcx_last_error_string()
    flag[0] = 3
    assert lib.mcx_poll_flag(ptr, 2, 0, 0) == L.MCX_OK
    flag[0] = 0

    def raise_later():
        time.sleep(0.02)
        flag[0] = 7

    th = threading.Thread(target=raise_later)
    th.start()
    assert lib.mcx_poll_flag(ptr, 7, 10 ** 7, 1000) == L.MCX_OK
    th.join()
    assert lib.mcx_poll_flag(None, 1, 1, 1) == L.MCX_ERR_INVALID_ARG
