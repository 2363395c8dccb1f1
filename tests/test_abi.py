"""The C ABI and host pieces that need no GPU: every function declared in include/*.h is
exported by libsofren2_gb300.so, the Python binding's sftg_tuning layout is the header's, and the
measured RCPPS/RSQRTPS tables reproduce the x86 instructions (checked against the instructions
themselves where the host is x86-64)."""
import ctypes as C
import os
import platform
import re
import subprocess
import tempfile

import numpy as np
import pytest

from sofren2_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header: str) -> set[str]:
    src = open(os.path.join(ROOT, "include", header)).read()
    src = src.split("#ifdef SFT_IMPL")[0]
    return set(re.findall(r"^(?:SFT_FUNC|int|void|uint64_t|double|const char\*)\s+[\w\s\*]*?\b((?:sft|sftg)_\w+)\s*\(", src, re.M))


@pytest.fixture(scope="module")
def lib_path():
    return build.build_library()


def test_library_exports_every_declared_symbol(lib_path):
    lib = C.CDLL(lib_path)
    declared = _declared("sofren2.h") | _declared("sftg.h")
    assert len(declared) > 60
    missing = [s for s in sorted(declared) if not hasattr(lib, s)]
    assert not missing, f"not exported: {missing}"


def test_scene_player_symbols(lib_path):
    lib = C.CDLL(lib_path)
    for s in ("sftx_scene_load", "sftx_scene_render", "sftx_scene_free", "sftx_scene_frame_count"):
        assert hasattr(lib, s)


def test_build_targets_sm103a_only():
    assert build.ARCH == "-gencode=arch=compute_103a,code=sm_103a"


@pytest.mark.skipif(platform.machine() != "x86_64", reason="needs the x86 RCPPS/RSQRTPS instructions")
def test_approx_tables_match_instructions():
    src = r'''
#include <immintrin.h>
#include <stdio.h>
#include <stdint.h>
#include <string.h>
#include "x86_approx_tables.h"
static const uint32_t R[2048] = SFT_X86_RCP_TABLE_INIT, Q[2048] = SFT_X86_RSQRT_TABLE_INIT;
static uint32_t rcp_t(uint32_t x){uint32_t s=x&0x80000000u,e=(x>>23)&255,m=x&0x7FFFFF;
 if(e==255)return m?(x|0x400000u):s; if(e==0)return s|0x7F800000u; if(e>=253)return s; return s|((253u-e)<<23)|R[m>>12];}
static uint32_t rsq_t(uint32_t x){uint32_t s=x&0x80000000u,e=(x>>23)&255,m=x&0x7FFFFF;
 if(e==255){if(m)return x|0x400000u;return s?0xFFC00000u:0u;} if(e==0)return s|0x7F800000u; if(s)return 0xFFC00000u;
 uint32_t t=Q[(e&1)*1024+(m>>13)]; int oe=((380-(int)e)>>1)+(int)(t>>23)-1; return ((uint32_t)oe<<23)|(t&0x7FFFFF);}
int main(void){uint64_t st=0x9E3779B97F4A7C15ull; unsigned bad=0;
 for(int i=0;i<(1<<22);i++){st^=st<<13;st^=st>>7;st^=st<<17; uint32_t x=(uint32_t)st; float f; memcpy(&f,&x,4);
  float r=_mm_cvtss_f32(_mm_rcp_ss(_mm_set_ss(f))), q=_mm_cvtss_f32(_mm_rsqrt_ss(_mm_set_ss(f))); uint32_t a,b; memcpy(&a,&r,4); memcpy(&b,&q,4);
  if(a!=rcp_t(x)||b!=rsq_t(x))bad++;} printf("%u\n",bad); return bad!=0;}
'''
    with tempfile.TemporaryDirectory() as td:
        c, exe = os.path.join(td, "t.c"), os.path.join(td, "t")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-O1", "-msse", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 0, f"{r.stdout.strip()} mismatching inputs"


def test_scene_generation_is_platform_independent():
    """Only IEEE add/sub/mul/div/sqrt feed the scenes: the deterministic sin/log stay within
    their polynomial error, and two generations give identical bytes."""
    from sofren2_gb300 import scenes
    x = np.linspace(-20, 20, 2001, dtype=np.float32)
    assert np.max(np.abs(scenes.dsin(x) - np.sin(x.astype(np.float64)))) < 2e-6
    y = np.linspace(0.01, 50, 999, dtype=np.float32)
    assert np.max(np.abs(scenes.dlog(y) - np.log(y.astype(np.float64)))) < 5e-6
    a = scenes.static_shapes_scene(64, 64, seed=3, n_spheres=2, n_cubes=1, tex_size=16).to_bytes()
    b = scenes.static_shapes_scene(64, 64, seed=3, n_spheres=2, n_cubes=1, tex_size=16).to_bytes()
    assert a == b


def test_serve_and_lane_calls_reject_bad_arguments(lib_path):
    """Argument checks that return before any GPU work: the serving loop without buffers or with
    an unknown mode, and the lane calls without a context."""
    lib = C.CDLL(lib_path)
    lib.sftx_serve.restype = C.c_int
    lib.sftx_serve.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint64, C.c_int, C.c_void_p, C.c_uint32,
                               C.c_void_p, C.c_void_p, C.c_void_p]
    dummy = (C.c_void_p * 1)()
    done = (C.c_uint64 * 1)()
    assert lib.sftx_serve(None, None, 0, 8, 1 << 30, 0, dummy, 8, done, None, None) == -1      # no scenes
    assert lib.sftx_serve(dummy, None, 0, 8, 1 << 30, 0, None, 8, done, None, None) == -1      # no colours
    assert lib.sftx_serve(dummy, None, 0, 8, 1 << 30, 0, dummy, 4, done, None, None) == -1     # ring < max_batch
    assert lib.sftx_serve(dummy, None, 0, 8, 1 << 30, 7, dummy, 8, done, None, None) == -1     # unknown mode
    for fn, args in (("sftg_frames_submit", (None, 1, None, 1, None, None)), ("sftg_lane_done", (None, 1)),
                     ("sftg_lane_wait", (None, 1))):
        f = getattr(lib, fn)
        f.restype = C.c_int
        assert f(*args) == -2, fn   # SFTG_E_ARG


def test_tuning_layout_matches_the_header(tmp_path):
    """runtime.TUNING_LAYOUT (the ctypes view of struct sftg_tuning) against the header, compiled:
    every field's offset and count, and the struct's size."""
    from sofren2_gb300.runtime import TUNING_LAYOUT
    cc = "gcc"
    names = [n for n, _ in TUNING_LAYOUT]
    prog = ["#include <stddef.h>", "#include <stdio.h>", '#include "sftg.h"', "int main(void) {",
            '    printf("%zu\\n", sizeof(sftg_tuning));']
    for n in names:
        prog.append(f'    printf("%zu %zu\\n", offsetof(sftg_tuning, {n}), sizeof(((sftg_tuning*)0)->{n}));')
    prog += ["    return 0;", "}"]
    src = tmp_path / "tuning_layout.c"
    src.write_text("\n".join(prog) + "\n")
    exe = tmp_path / "tuning_layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    assert int(out[0]) == 4 * sum(n for _, n in TUNING_LAYOUT)
    k = 0
    for (name, n), line in zip(TUNING_LAYOUT, out[1:]):
        off, size = map(int, line.split())
        assert (off, size) == (4 * k, 4 * n), name
        k += n
