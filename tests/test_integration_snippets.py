"""The C++ snippets of INTEGRATION.md that use the C ABI alone (Metropolis /
energy-redistribution options, the guided render, both batch schedulers)
compile against include/gbrt.h: a change of the header that the notes miss
fails here. The renderer's own types they touch (its cv::Mat film, its
boost::program_options map) are stood in for by two small structs; the
Renderer subclass snippet needs the renderer's headers and is left out."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PRELUDE = r'''
#include <cstdint>
#include <iostream>
#include <vector>
#include "gbrt.h"
struct Mat { template <class T> T* ptr(int) { return nullptr; } };          // cv::Mat
struct Opt { template <class T> T as() const { return T(); } };             // boost variable_value
struct Options { Opt operator[](const char*) const { return Opt(); } };     // boost variables_map
'''


def _blocks():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    return re.findall(r"```cpp\n(.*?)```", text, re.S)


@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_abi_snippets_compile(tmp_path):
    blocks = _blocks()
    chains = [b for b in blocks if "gbrt_render_mlt(" in b]
    guided = [b for b in blocks if "gbrt_render_guided(" in b]
    batch = [b for b in blocks if "gbrt_render_batch(" in b]
    fused = [b for b in blocks if "gbrt_render_batch_fused(" in b]
    assert len(chains) == len(guided) == len(batch) == len(fused) == 1
    src = PRELUDE + (
        "void chains(gbrt_scene* scene, gbrt_camera cam, gbrt_render_params p, Mat* film, const Options& vm) {\n"
        + chains[0] + "}\n"
        "void guided(gbrt_ctx* ctx, gbrt_scene* scene, gbrt_camera cam, Mat* film) {\n" + guided[0] + "}\n"
        "void batches(gbrt_ctx* ctx, int n, std::vector<gbrt_scene*> scenes, std::vector<gbrt_camera> cams,\n"
        "             std::vector<gbrt_render_params> params, std::vector<Mat> films) {\n"
        + batch[0] + fused[0] + "}\n")
    path = tmp_path / "snippets.cpp"
    path.write_text(src)
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Wno-unused-variable",
                        "-Wno-unused-but-set-variable", "-I", os.path.join(ROOT, "include"), str(path)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
