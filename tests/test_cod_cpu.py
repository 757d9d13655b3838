"""codeare's .cod matrix files (src/matrix/io/CODFile.hpp): the Python reader
and writer, their byte layout, and the plugin host's COD reader (no GPU)."""
import os
import struct
import subprocess

import numpy as np
import pytest


@pytest.mark.parametrize("dt", [np.float32, np.float64, np.complex64, np.complex128])
def test_round_trip_like_reference_test(tmp_path, dt):
    """A random 3 x 4 matrix of each type written and read back
    (src/matrix/io/tests/t_codeare.cpp:32-45)."""
    from codeare_gb300 import cod
    rng = np.random.default_rng(1)
    a = rng.standard_normal((4, 3))
    if np.issubdtype(dt, np.complexfloating):
        a = a + 1j * rng.standard_normal((4, 3))
    a = a.astype(dt)
    p = str(tmp_path / "test.cod")
    cod.write(p, a, "A", res=[0.5, 2.0])
    b, name, res = cod.read(p)
    assert name == "A" and b.dtype == a.dtype and b.shape == a.shape
    assert np.array_equal(a, b) and res == [0.5, 2.0]


def test_byte_layout(tmp_path):
    """Field order of CODFile::Write (CODFile.hpp:160-195)."""
    from codeare_gb300 import cod
    a = np.arange(6, dtype=np.complex64).reshape(2, 3)  # codeare 3 x 2
    p = tmp_path / "m.cod"
    cod.write(str(p), a, "sig")
    raw = p.read_bytes()
    assert struct.unpack_from("<i", raw, 0)[0] == 2
    assert struct.unpack_from("<Q", raw, 4)[0] == 2
    assert struct.unpack_from("<2Q", raw, 12) == (3, 2)
    assert struct.unpack_from("<2f", raw, 28) == (1.0, 1.0)
    assert struct.unpack_from("<Q", raw, 36)[0] == 3 and raw[44:47] == b"sig"
    assert np.array_equal(np.frombuffer(raw[47:47 + 48], np.complex64), a.ravel())
    assert raw[47 + 48:] == cod.DELIMITER and len(raw) == 47 + 48 + 32


def test_unknown_type_is_rejected(tmp_path):
    from codeare_gb300 import cod
    p = tmp_path / "bad.cod"
    p.write_bytes(struct.pack("<iQ", 9, 1))
    with pytest.raises(ValueError):
        cod.read(str(p))


def test_driver_reads_cod_inputs(tmp_path):
    """cgsense_run reads name=file.cod lists before it loads the plugin: with
    a plugin path that does not exist, readable inputs end in the dlopen
    failure (4) and a truncated file in the read failure (3)."""
    from codeare_gb300 import build, cod
    build.build()
    good = tmp_path / "s.cod"
    cod.write(str(good), np.ones((4, 8, 8), np.complex128), "sensitivities")
    w = tmp_path / "w.cod"
    cod.write(str(w), np.ones((1, 64), np.float64), "weights")
    xml = tmp_path / "c.xml"
    xml.write_text("<CGSENSE/>\n")
    missing = str(tmp_path / "nothing.so")
    r = subprocess.run([build.DRIVER, missing, str(xml), "sensitivities=%s,weights=%s" % (good, w),
                        str(tmp_path / "o.cod"), "image"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 4, r.stderr
    bad = tmp_path / "t.cod"
    bad.write_bytes(good.read_bytes()[:100])
    r = subprocess.run([build.DRIVER, missing, str(xml), "sensitivities=%s" % bad, str(tmp_path / "o.cod")],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 3, r.stderr
    r = subprocess.run([build.DRIVER, missing, str(xml), "sensitivities=%s" % good, str(tmp_path / "o.cod"),
                        "a", "b"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2
    assert os.path.exists(str(good))
