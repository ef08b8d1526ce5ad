"""CPU tests of the C ABI: the library loads, exports every symbol the header
declares, parses fish's options like the reference, and reports errors."""
import ctypes
import os
import re

import pytest

import _oracle as orc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "fishgpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text)) -
                  {"if", "sizeof", "defined"})


def test_library_exports_every_declared_symbol(built):
    import p4pdes_gb300 as fg
    lib = fg.load()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_sizes_match_the_header(built, tmp_path):
    """Compile a tiny C program against the header and compare sizeof/offsetof
    with the ctypes mirror."""
    import subprocess
    import p4pdes_gb300 as fg
    src = tmp_path / "sz.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "fishgpu.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(fishgpu_info),'
                   ' sizeof(fishgpu_ctx), sizeof(fishgpu_opts), sizeof(fishgpu_report),'
                   ' offsetof(fishgpu_opts, esteig), offsetof(fishgpu_report, dofs));return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    got = [int(v) for v in subprocess.run([str(exe)], stdout=subprocess.PIPE, text=True).stdout.split()]
    want = [ctypes.sizeof(fg.Info), ctypes.sizeof(fg.Ctx), ctypes.sizeof(fg.Opts), ctypes.sizeof(fg.Report),
            fg.Opts.esteig.offset, fg.Report.dofs.offset]
    assert got == want


def test_batch_and_server_structs_match_the_header(built, tmp_path):
    import subprocess
    import p4pdes_gb300 as fg
    src = tmp_path / "sz2.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "fishgpu.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(fishgpu_batch_opts),'
                   ' sizeof(fishgpu_batch_report), sizeof(fishgpu_server_opts), sizeof(fishgpu_server_result),'
                   ' offsetof(fishgpu_server_opts, rtol), offsetof(fishgpu_server_result, latency_ms));return 0;}\n')
    exe = tmp_path / "sz2"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    got = [int(v) for v in subprocess.run([str(exe)], stdout=subprocess.PIPE, text=True).stdout.split()]
    want = [ctypes.sizeof(fg.BatchOpts), ctypes.sizeof(fg.BatchReport), ctypes.sizeof(fg.ServerOpts),
            ctypes.sizeof(fg.ServerResult), fg.ServerOpts.rtol.offset, fg.ServerResult.latency_ms.offset]
    assert got == want


def test_minimal_structs_match_the_header(built, tmp_path):
    import subprocess
    import p4pdes_gb300 as fg
    src = tmp_path / "sz3.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "fishgpu.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(fishgpu_ms_ctx),'
                   ' sizeof(fishgpu_ms_opts), sizeof(fishgpu_ms_report), offsetof(fishgpu_ms_opts, ksp_rtol),'
                   ' offsetof(fishgpu_ms_report, area), offsetof(fishgpu_ms_report, total_ksp_its));return 0;}\n')
    exe = tmp_path / "sz3"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    got = [int(v) for v in subprocess.run([str(exe)], stdout=subprocess.PIPE, text=True).stdout.split()]
    want = [ctypes.sizeof(fg.MsCtx), ctypes.sizeof(fg.MsOpts), ctypes.sizeof(fg.MsReport),
            fg.MsOpts.ksp_rtol.offset, fg.MsReport.area.offset, fg.MsReport.total_ksp_its.offset]
    assert got == want


@pytest.mark.parametrize("args,grid,gs,deg", [
    ("", (3, 3), 0, 0),
    ("-da_refine 1 -ms_catenoid_c 2.0", (5, 5), 0, 0),
    ("-snes_grid_sequence 2 -ms_monitor -ms_quaddegree 2", (3, 3), 2, 2),
    ("-ms_quaddegree 2 -ms_monitor -da_refine 9", (1025, 1025), 0, 2),
    ("-ms_monitor", (3, 3), 0, 3),
    ("-ms_quaddegree 1", (3, 3), 0, 0),
])
def test_minimal_options(built, args, grid, gs, deg):
    import p4pdes_gb300 as fg
    o = fg.ms_options(args)
    assert (o.mx, o.my) == grid and o.grid_sequence == gs and o.monitor_degree == deg
    assert o.ctx.q == -0.5 and o.rtol == 1e-8 and o.ksp_rtol == 1e-5 and o.max_it == 50
    assert o.inner_block == 1 and o.inner_persist == -1 and o.vtail_points == 0


def test_minimal_inner_solve_options(built):
    import p4pdes_gb300 as fg
    o = fg.ms_options("-ms_inner_persist 0 -ms_vtail_points 4225 -ms_inner_block 0")
    assert o.inner_persist == 0 and o.vtail_points == 4225 and o.inner_block == 0


@pytest.mark.parametrize("args", ["-ms_catenoid_c 0.5", "-ms_problem nosuch", "-ms_quaddegree 4",
                                  "-ms_exact_init -ms_problem tent", "-ms_exact_init -ms_q 0"])
def test_minimal_bad_options(built, args):
    import p4pdes_gb300 as fg
    with pytest.raises(fg.FishError):
        fg.ms_options(args)


def test_server_options_for_a_request(built):
    import p4pdes_gb300 as fg
    o = fg.server_request_opts(3, 257)
    assert (o.mx, o.my, o.mz, o.mg_levels, o.ctx.problem) == (257, 257, 257, 8, fg.USER)
    est = fg.estimate_bytes(o)
    # mixed form: 6 FP64 + 9 FP32 fine-grid arrays, f, g, u on the host side, coarser levels
    assert 20 * 4 * 257 ** 3 < est < 40 * 4 * 257 ** 3
    bad = fg.server_request_opts(3, 257)
    bad.mx = 2
    assert fg.estimate_bytes(bad) == -1


def test_default_options_are_fish_defaults(built):
    import p4pdes_gb300 as fg
    o = fg.options([])
    assert o.ctx.dim == 2 and o.ctx.problem == fg.MANUEXP          # fish.c:140-141
    assert (o.mx, o.my) == (3, 3)                                   # 3x3 DMDA, fish.c:203-205
    assert o.initial_gonboundary == 1 and o.initial_type == 0       # fish.c:142-143
    assert o.rtol == 1e-5 and o.max_it == 10000 and o.smooth_its == 2
    assert list(o.esteig) == [0.0, 0.1, 0.0, 1.1]


def test_build_options_parse_and_default(built):
    """The library's options beside fish's: precision form, inner tolerances,
    graph shape, device-side loop, fused post-smoother, paired FP64 updates,
    cooperative V-cycle tail."""
    import p4pdes_gb300 as fg
    o = fg.options([])
    assert o.device_loop == 1 and o.fuse_smooth == 0 and o.precision == fg.FP64
    assert o.pair_y == 1 and o.coop_tail == 0
    o2 = fg.options(["-fsh_pair_y", "0", "-fsh_coop_tail", "-1"])
    assert o2.pair_y == 0 and o2.coop_tail == -1
    o = fg.options("-fsh_precision mixed -fsh_inner_rtol 1e-7 -fsh_inner_max_it 50 -fsh_outer_max_it 9 "
                   "-fsh_graph_iters 6 -fsh_device_loop 0 -fsh_fuse_smooth 1")
    assert o.precision == fg.MIXED and o.inner_rtol == 1e-7 and o.inner_max_it == 50 and o.outer_max_it == 9
    assert o.graph_iters == 6 and o.device_loop == 0 and o.fuse_smooth == 1


@pytest.mark.parametrize("args,grid,levels", [
    ("-fsh_dim 2 -da_refine 7 -pc_type mg", (257, 257, 1), 8),
    ("-fsh_dim 3 -da_refine 8", (513, 513, 513), 9),
    ("-fsh_dim 1 -da_refine 3", (17, 1, 1), 4),
    ("-fsh_dim 3 -da_refine 7 -pc_mg_levels 6", (257, 257, 257), 6),
    ("-fsh_dim 2 -da_grid_x 5 -da_grid_y 9 -da_refine 2", (17, 33, 1), 3),
])
def test_grid_and_levels_from_options(built, args, grid, levels):
    import p4pdes_gb300 as fg
    o = fg.options(args)
    d = o.ctx.dim
    assert (o.mx, o.my if d >= 2 else 1, o.mz if d >= 3 else 1) == grid
    assert o.mg_levels == levels
    oo = orc.options(args)
    assert (oo.grid.mx, oo.grid.my, oo.grid.mz) == grid and oo.mg_levels == levels


@pytest.mark.parametrize("args,code", [
    ("-fsh_dim 4", 1),
    ("-fsh_cx -1", 1),                                  # fish.c:188-190
    ("-fsh_problem manuexp -fsh_cx 2", 1),              # fish.c:191-193
    ("-fsh_problem nosuch", 1),
    ("-pc_type ilu", 7),
    ("-mg_levels_pc_type sor", 7),
    ("-ksp_type gmres", 7),
    ("-da_refine", 1),
])
def test_invalid_options_are_rejected(built, args, code):
    import p4pdes_gb300 as fg
    with pytest.raises(fg.FishError) as e:
        fg.options(args)
    assert e.value.code == code


def test_golden_option_sets_parse(built):
    import json
    import p4pdes_gb300 as fg
    for rec in json.load(open(os.path.join(ROOT, "tests", "golden", "fish_goldens.json"))):
        o = fg.options(rec["args"])
        oo = orc.options(rec["args"])
        assert (o.mx, o.ctx.problem, o.ctx.dim) == (oo.grid.mx, oo.grid.problem, oo.grid.dim)
        assert abs(o.rtol - oo.rtol) == 0


def test_status_strings(built):
    import p4pdes_gb300 as fg
    lib = fg.load()
    for code in range(0, 9):
        assert lib.fishgpu_strerror(code)
    assert fg.reason_name(2) == "CONVERGED_RTOL" and fg.reason_name(-3) == "DIVERGED_ITS"


def test_solver_without_device_reports_nodevice(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    import p4pdes_gb300 as fg
    with pytest.raises(fg.FishError) as e:
        fg.Solver(fg.options("-fsh_dim 2 -da_refine 2"))
    assert e.value.code == 8


def test_null_arguments_are_rejected(built):
    import p4pdes_gb300 as fg
    lib = fg.load()
    inf = fg.Info()
    ctx = fg.Ctx()
    assert lib.Poisson2DFunctionLocal_gpu(None, None, None, None, None) == 1
    assert lib.Poisson3DOperatorApply_gpu(ctypes.byref(inf), None, None, None, ctypes.byref(ctx), None) == 1
    assert lib.fishgpu_solver_create(None, None, None) == 1
