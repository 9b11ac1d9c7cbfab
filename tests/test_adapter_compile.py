"""The drop-in adapter (illum-rt_gb300/adapter/gb300_rt.h, the wf::cuda::batch_rt subclass a
maintainer adds to the reference's CUDA platform) compiles against the reference's own headers:
its overrides match wf::cuda::batch_rt (rt/cuda/base.h:403-429), and registering and selecting it
the way platform::platform and platform::interprete do (register_batch_rt,
libgi/wavefront-rt.h:48; rt/cuda/platform.cpp:34-56, 102-131) type-checks. CPU only; skipped
where the reference checkout is absent."""
import importlib.util
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBE = r'''
#include "gb300.h"
#include "platform.h"

// A platform that registers and selects the adapter as rt/cuda/platform.cpp does for its own
// tracers; only compiled, never constructed.
struct gb300_platform_probe : public wf::cuda::platform {
    void register_gb300() {
        register_batch_rt("gb300",, wf::cuda::gb300_rt("while-while"));
        register_batch_rt("gb300-persistent",, wf::cuda::gb300_rt("persistent-speculative-while-while"));
    }
    wf::cuda::batch_rt *select_gb300() { return dynamic_cast<wf::cuda::batch_rt *>(select("gb300")); }
};

// The adapter is a concrete wf::cuda::batch_rt and a wf::batch_ray_tracer.
static_assert(!std::is_abstract<wf::cuda::gb300_rt>::value, "gb300_rt must implement compute_hit");
static_assert(std::is_base_of<wf::cuda::batch_rt, wf::cuda::gb300_rt>::value, "not a batch_rt");
static_assert(std::is_base_of<wf::batch_ray_tracer, wf::cuda::gb300_rt>::value, "not a batch_ray_tracer");
// grt_hit is the reference's tri_is, byte for byte, so buffers pass through unconverted.
static_assert(sizeof(grt_hit) == sizeof(wf::cuda::tri_is), "hit record size");
static_assert(offsetof(grt_hit, ref) == offsetof(wf::cuda::tri_is, ref), "hit record layout");
'''


def _reference_dir():
    d = os.environ.get("GRT_REFERENCE_DIR")
    if not d:
        spec = importlib.util.spec_from_file_location("grt_oracle_build", os.path.join(ROOT, "oracle", "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        d = mod.REFERENCE_CHECKOUT
    return d if os.path.exists(os.path.join(d, "rt", "cuda", "base.h")) else None


def _cuda_include():
    nvcc = shutil.which("nvcc")
    for base in ([os.path.dirname(os.path.dirname(nvcc))] if nvcc else []) + ["/usr/local/cuda"]:
        inc = os.path.join(base, "include")
        if os.path.exists(os.path.join(inc, "cuda_runtime_api.h")):
            return inc
    return None


def test_adapter_compiles_against_reference_headers(tmp_path):
    ref, cuda_inc = _reference_dir(), _cuda_include()
    if ref is None or cuda_inc is None:
        pytest.skip("reference checkout or CUDA headers absent")
    # the adapter as a maintainer places it: rt/cuda/gb300.h next to base.h
    shutil.copy(os.path.join(ROOT, "illum-rt_gb300", "adapter", "gb300_rt.h"), tmp_path / "gb300.h")
    (tmp_path / "probe.cpp").write_text(PROBE)
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-I" + str(tmp_path), "-I" + ref, "-I" + os.path.join(ref, "rt", "cuda"),
           "-I" + os.path.join(ref, "libgi"), "-I" + os.path.join(ROOT, "oracle", "shim"),
           "-I" + os.path.join(ROOT, "include"), "-I" + cuda_inc, str(tmp_path / "probe.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


def test_adapter_rejects_a_wrong_override(tmp_path):
    """The check has teeth: the same compile fails when the adapter's compute_hit does not
    match the reference's signature."""
    ref, cuda_inc = _reference_dir(), _cuda_include()
    if ref is None or cuda_inc is None:
        pytest.skip("reference checkout or CUDA headers absent")
    src = open(os.path.join(ROOT, "illum-rt_gb300", "adapter", "gb300_rt.h")).read()
    bad = src.replace("void compute_hit(bool anyhit) override", "void compute_hit(int anyhit) override")
    assert bad != src
    (tmp_path / "gb300.h").write_text(bad)
    (tmp_path / "probe.cpp").write_text(PROBE)
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-I" + str(tmp_path), "-I" + ref, "-I" + os.path.join(ref, "rt", "cuda"),
           "-I" + os.path.join(ref, "libgi"), "-I" + os.path.join(ROOT, "oracle", "shim"),
           "-I" + os.path.join(ROOT, "include"), "-I" + cuda_inc, str(tmp_path / "probe.cpp")]
    assert subprocess.run(cmd, capture_output=True, text=True).returncode != 0
