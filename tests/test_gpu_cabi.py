"""OAK's C interface (oak_init / oak_assim / oak_done): context lifecycle and status codes."""
import ctypes
import os

import pytest

pytestmark = pytest.mark.gpu


def test_oak_entry_points(oakg, tmp_path):
    L = oakg.lib()
    L.oak_init(b"/nonexistent/assim.init")
    assert L.oakg_last_status() == oakg.ERR_INIT
    init = tmp_path / "assim.init"
    init.write_text("runtype = 2\\nschemetype = 1\\n")
    L.oak_init(str(init).encode())
    assert L.oakg_last_status() == 0
    L.oak_assim(1, 4, 3, None, None)
    assert L.oakg_last_status() == oakg.ERR_NOTIMPL
    buf = ctypes.create_string_buffer(512)
    L.oakg_last_error(buf, 512)
    assert b"oakg_ens_locanalysis" in buf.value
    L.oak_done()
    assert L.oakg_last_status() == 0
