"""C++ facade (acts_gb300/host/ActsPlugins/CudaKalman.hpp): compiles on CPU;
per-track and batched fits through it on the GPU agree bit for bit; track
finding through it finds each seed's own hits."""
import os
import subprocess

import pytest

from acts_gb300.build import INCLUDE, LIBDIR, build_cuda, build_generator

HERE = os.path.dirname(os.path.abspath(__file__))
HOST = os.path.join(os.path.dirname(HERE), "acts_gb300", "host")


def _compile(out):
    build_cuda()
    build_generator()
    cmd = ["g++", "-std=c++17", "-O1", "-I" + INCLUDE, "-I" + HOST,
           os.path.join(HERE, "cpp", "test_facade.cpp"), "-o", out, "-L" + LIBDIR,
           "-lcudakalman", "-lckgen", "-Wl,-rpath," + LIBDIR]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout


def test_facade_compiles(tmp_path):
    _compile(str(tmp_path / "test_facade"))


@pytest.mark.gpu
def test_facade_runs_on_gpu(tmp_path):
    exe = str(tmp_path / "test_facade")
    _compile(exe)
    r = subprocess.run([exe], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout
    assert "facade ok" in r.stdout
    assert "findTracks ok" in r.stdout
