"""The upside command line of libupside.so (upside_main) without a GPU: the
reference's arguments (src/main.cpp:428-529) are parsed, missing required
ones and unknown ones are errors with return code 1 (as TCLAP reports them),
and options the GPU driver does not support are refused before any device
work.  Runs of the driver are in test_gpu_driver.py."""
import ctypes
import os
import subprocess

from conftest import GOLDEN, ROOT

PKG = os.path.join(ROOT, "upside2-md_gb300")


def _main(args):
    L = ctypes.CDLL(os.path.join(PKG, "libupside.so"))
    L.upside_main.restype = ctypes.c_int
    L.upside_main.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p), ctypes.c_int]
    argv = ["upside"] + list(args)
    arr = (ctypes.c_char_p * len(argv))(*[a.encode() for a in argv])
    return L.upside_main(len(argv), arr, 0)


def test_arguments(built, capfd):
    cfg = os.path.join(GOLDEN, "chig.up")
    assert _main(["--help"]) == 0
    assert "--frame-interval" in capfd.readouterr().out
    assert _main(["--duration", "1", cfg]) == 1
    assert "Required argument missing for argument frame-interval" in capfd.readouterr().err
    assert _main(["--frame-interval", "1", cfg]) == 1
    assert "duration" in capfd.readouterr().err
    assert _main(["--duration", "1", "--frame-interval", "1"]) == 1
    assert "config_files" in capfd.readouterr().err
    assert _main(["--duration", "1", "--frame-interval", "1", "--no-such-option", cfg]) == 1
    assert "--no-such-option" in capfd.readouterr().err
    assert _main(["--duration", "x1", "--frame-interval", "1", cfg]) == 1
    assert "invalid float" in capfd.readouterr().err
    assert _main(["--duration", "1", "--frame-interval"]) == 1
    assert "Missing a value" in capfd.readouterr().err
    for extra, word in ((["--integrator", "leapfrog"], "integrator"),
                        (["--curvature-changer-interval", "2"], "curvature"),
                        (["--potential-deriv-agreement"], "deriv-agreement"),
                        (["--log-level", "loud"], "log-level")):
        assert _main(["--duration", "1", "--frame-interval", "1"] + extra + [cfg]) == 1, extra
        assert word in capfd.readouterr().err, extra
    assert _main(["--duration", "1", "--frame-interval", "1", "--temperature", "1,2", cfg]) == 1
    assert "Received 2 temperatures but have 1 systems" in capfd.readouterr().err
    assert _main(["--duration", "1", "--frame-interval", "1", os.path.join(ROOT, "no_such.up")]) == 1
    assert "Unable to open configuration file" in capfd.readouterr().err


def test_executable(built):
    exe = os.path.join(PKG, "upside")
    r = subprocess.run([exe, "--duration", "1"], capture_output=True, text=True)
    assert r.returncode == 1 and "frame-interval" in r.stderr
    r = subprocess.run([exe, "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "USAGE" in r.stdout
