"""The Java binding committed as source (openpixi_gb300/jni): OpixiJNI.c calls
only entry points that include/opixi.h declares and libopixi_gpu.so exports;
its JNI exports and the native methods of Opixi.java match one for one; and
the C compiles (gcc, with a test-only stand-in for the JNI types since no JDK
exists here).  No device is used."""
import os
import re
import shutil
import subprocess

import pytest

from test_abi_cpu import header_symbols

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
JNI = os.path.join(ROOT, "openpixi_gb300", "jni")
SHIM = os.path.join(JNI, "OpixiJNI.c")
JAVA = os.path.join(JNI, "org", "openpixi", "pixi", "gpu", "Opixi.java")


def shim_calls():
    txt = re.sub(r"/\*.*?\*/", "", open(SHIM).read(), flags=re.S)
    return sorted(set(re.findall(r"\b(opx_[a-z_]+)\s*\(", txt)))


def test_shim_calls_are_declared_and_exported(native):
    calls = shim_calls()
    declared = set(header_symbols())
    assert calls and set(calls) <= declared, set(calls) - declared
    for name in calls:
        assert hasattr(native, name), name
    # the entry points a drop-in needs are bound
    for need in ("opx_download", "opx_particles_upload", "opx_particles_download", "opx_cpic_phases",
                 "opx_projected_energy", "opx_objective_gradient", "opx_host_alloc"):
        assert need in calls, need


def test_jni_exports_match_java_natives():
    c = open(SHIM).read()
    exports = set(re.findall(r"Java_org_openpixi_pixi_gpu_Opixi_([A-Za-z0-9]+)\s*\(", c))
    java = open(JAVA).read()
    natives = set(re.findall(r"public static native [\w\[\]]+ (\w+)\(", java))
    assert exports and exports == natives, (exports ^ natives)


def test_shim_compiles():
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("no gcc")
    r = subprocess.run([gcc, "-std=c11", "-Wall", "-Wextra", "-Werror", "-fsyntax-only",
                        "-I", os.path.join(ROOT, "tests", "jni_stub"), "-I", os.path.join(ROOT, "include"), SHIM],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
