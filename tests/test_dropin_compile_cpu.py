"""The C++ drop-in headers compile in libgran's driver compositions without a GPU (running them
needs one: tests/test_gpu_cpp_dropin.py, tests/test_gpu_unary.py): libgran's hamaker and sintered
tests, the custom step-handler tutorial, the writer, and a __device__ unary functor (nvcc)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include", "libgran_gb300")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


@pytest.mark.parametrize("src", ["dropin_hamaker.cpp", "dropin_sintered.cpp", "dropin_tutorial.cpp", "dropin_writer.cpp"])
def test_dropin_driver_compiles(tmp_path, src):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    r = subprocess.run(["g++", "-std=c++17", "-O0", "-fsyntax-only", "-Wall", "-I" + INC,
                        "-I" + os.path.join(CUDA, "include"), os.path.join(ROOT, "tests", "cpp", src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_device_functor_driver_compiles(tmp_path):
    nvcc = os.path.join(CUDA, "bin", "nvcc")
    if not os.path.exists(nvcc):
        pytest.skip("no nvcc")
    r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-I" + INC,
                        "-I" + os.path.join(ROOT, "include"), "-c",
                        os.path.join(ROOT, "tests", "cpp", "device_unary_central.cu"), "-o",
                        str(tmp_path / "d.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_custom_binary_functor_is_rejected_at_compile_time(tmp_path):
    """A binary functor without a GPU implementation fails to compile with a clear message."""
    if not shutil.which("g++"):
        pytest.skip("no g++")
    src = tmp_path / "bad.cpp"
    src.write_text('''
#include <libgran/contact_force/contact_force.h>
#include <libgran/granular_system/granular_system.h>
#include <vector>
struct v3 { double c[3]; v3() : c{0, 0, 0} {} v3(double a, double b, double d) : c{a, b, d} {}
            double operator[](int k) const { return c[k]; } };
struct my_functor { std::pair<v3, v3> operator()(size_t, size_t, std::vector<v3> const &, std::vector<v3> const &,
                                                  std::vector<v3> const &, std::vector<v3> const &, double) { return {}; } };
int main() {
    my_functor f;
    binary_force_functor_container<v3, double, my_functor> b{f};
    unary_force_functor_container<v3, double> u;
    rotational_step_handler<std::vector<v3>, v3> h;
    std::vector<v3> x(2);
    granular_system<v3, double, rotational_velocity_verlet_half, rotational_step_handler,
                    binary_force_functor_container<v3, double, my_functor>,
                    unary_force_functor_container<v3, double>> s(x, x, x, x, 0.0, v3(), 0.0, h, b, u);
    return 0;
}
''')
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I" + INC, "-I" + os.path.join(CUDA, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode != 0
    assert "no GPU implementation" in r.stderr
