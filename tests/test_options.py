"""Options file parsing (options.cu:12-53 semantics) through the C ABI, and the
driver's handling of a missing options file.  No GPU needed."""
import os
import subprocess

import pytest


def write(tmp_path, text, name="gpu.conf"):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_reference_gpu_conf(gdlib, tmp_path):
    o = gdlib.load_options(write(tmp_path, "nx = 16\nny = 16\nnz = 16\n\nnpx = 256\n"))
    assert o == {"nx": 16, "ny": 16, "nz": 16, "nyz": 256, "nxyz": 4096, "npx": 256}


def test_comments_whitespace_unknown_keys(gdlib, tmp_path):
    text = "# grid\n  nx=20  \n\tny =\t12\nnz= 8 # std::stoi reads the leading integer\nfoo = bar\n#npx = 7\nnpx = 64\n"
    o = gdlib.load_options(write(tmp_path, text))
    assert (o["nx"], o["ny"], o["nz"], o["npx"]) == (20, 12, 8, 64)


def test_partial_numeric_values_like_stoi(gdlib, tmp_path):
    o = gdlib.load_options(write(tmp_path, "nx = 20abc\nny=12\nnz=8\nnpx=3\nextra = 5\n# nx = 99\n"))
    assert (o["nx"], o["ny"], o["nz"], o["npx"], o["nxyz"]) == (20, 12, 8, 3, 20 * 12 * 8)


def test_missing_file(gdlib, tmp_path):
    with pytest.raises(gdlib.GDError) as e:
        gdlib.load_options(str(tmp_path / "nope.conf"))
    assert e.value.code == 6
    assert "Can't open" in str(e.value)


def test_non_numeric_value(gdlib, tmp_path):
    with pytest.raises(gdlib.GDError) as e:
        gdlib.load_options(write(tmp_path, "nx = sixteen\n"))
    assert e.value.code == 1


def test_driver_missing_options_file(gdlib, tmp_path):
    exe = os.path.join(os.path.dirname(gdlib.library_path()), "gd_determ")
    r = subprocess.run([exe, str(tmp_path / "missing.conf")], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 2
    assert "Can't open" in r.stderr
