"""The in-tree Mode::CUDA adaptor (pipeline_gb300/cpp/reference_backend/dp/culling/cuda)
compiles against the reference's own headers and links against the reference's culling
objects plus libdpcull.so.  Runs where the reference sources exist; the culls themselves
need a GPU as well, and the GPU host has no copy of the reference sources, so where the
two do not meet the driver stops at the backend's "no CUDA device" error."""
import subprocess

import pytest

import oracle
from conftest import ROOT

REF = oracle.REF_SRC
pytestmark = pytest.mark.skipif(not REF.is_dir(), reason="reference sources not present")

MAIN = r"""
#include <dp/culling/cuda/Manager.h>
#include <dp/culling/cpu/Manager.h>
#include <cstdio>
#include <cstring>
#include <memory>
#include <random>
#include <stdexcept>
#include <vector>
using namespace dp::culling;
// The same scene in the Mode::CUDA adaptor and in the reference CPU manager: three culls
// (a first frame, a frame after some matrices were marked changed, a frame after some
// boxes changed), every changed list compared.
int main() {
  try {
    std::unique_ptr<Manager> gpu(cuda::Manager::create(0));
    std::unique_ptr<Manager> cpu(cpu::Manager::create());
    const size_t n = 5000, nm = 300;
    std::mt19937 rng(7);
    std::uniform_real_distribution<float> u(-1.f, 1.f);
    std::vector<dp::math::Mat44f> mats(nm);
    for (auto& m : mats) {
      m = dp::math::cIdentity44f;
      for (int c = 0; c < 3; ++c) m[3][c] = 50.f * u(rng);
    }
    Manager* ms[2] = {gpu.get(), cpu.get()};
    GroupSharedPtr g[2];
    ResultSharedPtr r[2];
    std::vector<ObjectSharedPtr> objs[2];
    for (int k = 0; k < 2; ++k) {
      g[k] = ms[k]->groupCreate();
      r[k] = ms[k]->groupCreateResult(g[k]);
    }
    std::mt19937 rb(9);
    for (size_t i = 0; i < n; ++i) {
      dp::math::Vec3f lo(u(rb), u(rb), u(rb)), hi(lo[0] + 1.f, lo[1] + 2.f, lo[2] + 0.5f);
      size_t t = rb() % nm;
      for (int k = 0; k < 2; ++k) {
        ObjectSharedPtr o = ms[k]->objectCreate(PayloadSharedPtr());
        ms[k]->objectSetBoundingBox(o, dp::math::Box3f(lo, hi));
        ms[k]->objectSetTransformIndex(o, t);
        ms[k]->groupAddObject(g[k], o);
        objs[k].push_back(o);
      }
    }
    dp::math::Mat44f vp = dp::math::cIdentity44f;
    vp[0][0] = 0.02f; vp[1][1] = 0.03f; vp[2][2] = 0.01f;
    for (int frame = 0; frame < 3; ++frame) {
      if (frame == 1) {  // animate some transforms, as the patched CullingImpl reports them
        for (size_t i = 0; i < nm; i += 7) {
          mats[i][3][0] += 40.f;
          for (int k = 0; k < 2; ++k) ms[k]->groupMatrixChanged(g[k], i);
        }
      }
      if (frame == 2) {  // move some boxes
        for (size_t i = 0; i < n; i += 11) {
          dp::math::Box3f b(dp::math::Vec3f(30.f, 0.f, 0.f), dp::math::Vec3f(31.f, 1.f, 1.f));
          for (int k = 0; k < 2; ++k) ms[k]->objectSetBoundingBox(objs[k][i], b);
        }
      }
      size_t sizes[2];
      std::vector<size_t> idx[2];
      for (int k = 0; k < 2; ++k) {
        ms[k]->groupSetMatrices(g[k], mats.data(), nm, sizeof(mats[0]));
        ms[k]->cull(g[k], r[k], vp);
        for (auto const& o : ms[k]->resultGetChanged(r[k]))
          for (size_t i = 0; i < n; ++i) if (objs[k][i] == o) { idx[k].push_back(i); break; }
        sizes[k] = idx[k].size();
      }
      if (idx[0] != idx[1]) { std::printf("mismatch frame %d: %zu vs %zu\n", frame, sizes[0], sizes[1]); return 3; }
      for (size_t i = 0; i < n; i += 97)
        if (ms[0]->resultObjectIsVisible(r[0], objs[0][i]) != ms[1]->resultObjectIsVisible(r[1], objs[1][i])) {
          std::printf("visibility mismatch frame %d object %zu\n", frame, i); return 4; }
      std::printf("frame %d changed %zu\n", frame, sizes[0]);
    }
    std::printf("ok scene\n");
  } catch (std::exception const& e) {
    std::printf("error: %s\n", e.what());
    return 2;
  }
  return 0;
}
"""


def test_adaptor_compiles_and_links(tmp_path):
    from pipeline_gb300 import build

    build.build_cuda()
    oracle.build(with_reference=True)
    main = tmp_path / "main.cpp"
    main.write_text(MAIN)
    rb = ROOT / "pipeline_gb300" / "cpp" / "reference_backend"
    lib = ROOT / "pipeline_gb300" / "_lib"
    exe = tmp_path / "adaptor"
    cmd = ["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-I", str(REF), "-I", str(ROOT / "oracle" / "ref_shim"),
           "-I", str(ROOT / "include"), "-I", str(rb), str(rb / "dp/culling/cuda/src/ManagerImpl.cpp"), str(main),
           "-o", str(exe), "-L", str(oracle.REF_LIB.parent), "-ldpref", "-L", str(lib), "-ldpcull",
           f"-Wl,-rpath,{oracle.REF_LIB.parent}:{lib}", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    # With a GPU every changed list equals the reference CPU manager's; without one the
    # backend reports an error instead of falling back to the CPU.
    assert ("ok scene" in r.stdout) or ("no CUDA device" in r.stdout), r.stdout + r.stderr


def test_xbar_patch_applies_and_compiles(tmp_path):
    """pipeline_gb300/cpp/reference_backend/xbar_culling_cuda.patch (Mode::CUDA in the
    culling-mode switch and the transform observer attached, dp/sg/xbar/culling/src/
    CullingImpl.cpp:52-63,102,217-224) applies to the reference's files and the patched
    CullingImpl.cpp compiles against the reference headers and the adaptor's Manager.h."""
    rel = ["dp/sg/xbar/culling/src/CullingImpl.cpp", "dp/sg/xbar/culling/inc/CullingImpl.h"]
    for f in rel:
        (tmp_path / f).parent.mkdir(parents=True, exist_ok=True)
        (tmp_path / f).write_bytes((REF / f).read_bytes())
    patch = ROOT / "pipeline_gb300" / "cpp" / "reference_backend" / "xbar_culling_cuda.patch"
    r = subprocess.run(["patch", "-p1", "-d", str(tmp_path), "-i", str(patch)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    src = (tmp_path / rel[0]).read_text()
    assert "case dp::culling::Mode::CUDA:" in src and "attach( &m_transformObserver )" in src
    rb = ROOT / "pipeline_gb300" / "cpp" / "reference_backend"
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-w", "-I", str(tmp_path), "-I", str(rb), "-I", str(REF),
                        "-I", str(ROOT / "oracle" / "ref_shim"), "-I", str(ROOT / "include"), str(tmp_path / rel[0])],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
