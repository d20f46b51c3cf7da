"""OAK's C interface (oak_init / oak_assim / oak_done): context lifecycle and status codes."""
import ctypes
import os

import pytest

pytestmark = pytest.mark.gpu


def test_oak_entry_points(oakg, tmp_path):
    """The reference's C entry points through ctypes: a missing init file, a free run
    (runtype 0: Ea = Ef), NULL arrays, an assimilation setup without the model's keys."""
    import numpy as np
    L = oakg.lib()
    L.oak_init(b"/nonexistent/assim.init")
    assert L.oakg_last_status() == oakg.ERR_INIT
    init = tmp_path / "free.init"
    init.write_text("runtype = 0" + chr(10))
    L.oak_init(str(init).encode())
    assert L.oakg_last_status() == 0
    Ef = np.asfortranarray(np.arange(12.0).reshape(4, 3))
    Ea = np.zeros_like(Ef, order="F")
    L.oak_assim(1, 4, 3, Ef.ctypes.data_as(ctypes.c_void_p), Ea.ctypes.data_as(ctypes.c_void_p))
    assert L.oakg_last_status() == 0 and np.array_equal(Ea, Ef)
    L.oak_assim(1, 4, 3, None, None)
    assert L.oakg_last_status() == oakg.ERR_ARGS
    init = tmp_path / "assim.init"
    init.write_text("runtype = 2" + chr(10) + "schemetype = 1" + chr(10))
    L.oak_init(str(init).encode())
    assert L.oakg_last_status() == oakg.ERR_INIT
    buf = ctypes.create_string_buffer(512)
    L.oakg_last_error(buf, 512)
    assert b"Model.mask" in buf.value
    L.oak_done()
    assert L.oakg_last_status() == 0

