"""CPU tests of the C ABI boundary: the library loads, exports every symbol the
public headers declare, and rejects bad arguments before touching a GPU."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for hdr in ("convGemm.h", "convgemm_gpu.h"):
        src = open(os.path.join(ROOT, "include", hdr)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b([A-Za-z_]\w*)\s*\([^;{]*\)\s*;", src, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_reference_entry_points():
    names = declared_functions()
    for n in ("alloc_pack_buffs", "sconvGemmNHWC", "sconvGemmNHWC_back", "sconvGemmNCHW", "sconvGemmNCHW_back"):
        assert n in names


def test_library_exports_every_declared_symbol(cglib):
    L = cglib.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_drop_in_header_compiles_as_c(tmp_path):
    """convGemm.h is usable from plain C (it brings its own <stdbool.h>)."""
    import subprocess
    src = tmp_path / "t.c"
    src.write_text('#include "convGemm.h"\nint main(void){float*a,*b;return alloc_pack_buffs(&a,&b);}\n')
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"), "-c",
                        str(src), "-o", str(tmp_path / "t.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_alloc_pack_buffs_needs_no_gpu(cglib):
    rc, a, b = cglib.alloc_pack_buffs()
    assert rc == 0 and a is None and b is None


@pytest.mark.parametrize("bad", [
    dict(b=0), dict(kh=9), dict(vstride=0), dict(hdil=0), dict(vpad=-1), dict(c=0),
])
def test_invalid_geometry_rejected_without_gpu(cglib, bad):
    args = dict(b=1, h=5, w=5, c=3, kn=4, kh=3, kw=3, vpad=0, hpad=0, vstride=1, hstride=1, vdil=1, hdil=1)
    args.update(bad)
    s = cglib.Shape(*[args[k] for k in ("b", "h", "w", "c", "kn", "kh", "kw", "vpad", "hpad", "vstride",
                                        "hstride", "vdil", "hdil")])
    L = cglib.lib()
    st = L.convgemm_fwd_f32(0, ctypes.byref(s), 1, 1, 1, None, None)   # non-NULL dummies: never dereferenced
    assert st == 1, cglib.last_error()
    assert cglib.last_error()[0] == 1
    assert L.convgemm_wgrad_f32_workspace_size(ctypes.byref(s)) == 0


def test_dropin_records_error_instead_of_crashing(cglib):
    """The void drop-in reports bad geometry through the last-error API."""
    with pytest.raises(cglib.ConvGemmError) as ei:
        cglib.sconvGemmNHWC("N", 1, 2, 2, 3, 4, 5, 5, 0, 0, 1, 1, 1, 1, None, None, None)
    assert ei.value.status == 1


def test_batchnorm_needs_all_parameters(cglib):
    s = cglib.Shape.of(1, 5, 5, 3, 4, 3, 3)
    e = cglib.Epilogue(None, 1, None, None, None, 0)
    st = cglib.lib().convgemm_fwd_f32(0, ctypes.byref(s), 1, 1, 1, ctypes.byref(e), None)
    assert st == 1 and "batch-norm" in cglib.last_error()[1]


def test_workspace_size_query(cglib):
    s = cglib.Shape.of(2, 10, 10, 4, 8, 3, 3, 1, 1)
    n = cglib.wgrad_f32_workspace_size(s)
    nblocks = -(-(2 * 10 * 10) // 384)
    assert n == 4 * nblocks * 36 * 8


def test_group_prepare_rejects_bad_arguments_without_gpu(cglib):
    from convgemm_gb300 import tc
    L = cglib.lib()
    tiles = ctypes.c_int(0)
    assert L.convgemm_group_prepare(0, None, None, 0, ctypes.byref(tiles)) == 1
    s = cglib.Shape.of(1, 8, 8, 12, 16, 3, 3, 1, 1)   # c % 8 != 0
    assert L.convgemm_group_weights_size(ctypes.byref(s)) == 0
    conv = tc.GroupConv(s, 16, 16, 16, None, None, 0, 0)
    buf = ctypes.create_string_buffer(L.convgemm_group_table_size(1) + 64)
    addr = (ctypes.addressof(buf) + 63) // 64 * 64
    st = L.convgemm_group_prepare(1, ctypes.addressof(conv), addr, L.convgemm_group_table_size(1), ctypes.byref(tiles))
    assert st != 0 and "c % 8" in cglib.last_error()[1]
    assert L.convgemm_group_table_size(4) == 4 * L.convgemm_group_table_size(1) > 0


def test_tune_table_validation_without_gpu(cglib):
    from convgemm_gb300 import tc
    s = cglib.Shape.of(2, 8, 8, 64, 64, 3, 3, 1, 1)
    L = cglib.lib()
    assert L.convgemm_tune_set(9, ctypes.byref(s), 64, 0) == 1
    assert L.convgemm_tune_set(tc.TUNE_FWD, ctypes.byref(s), 96, 0) == 1
    assert L.convgemm_tune_set(tc.TUNE_FWD, ctypes.byref(s), 64, 4) == 1      # splits: weight gradient only
    assert L.convgemm_tune_set(tc.TUNE_FWD, ctypes.byref(s), 64, 3) == 1
    assert L.convgemm_tune_set(tc.TUNE_DGRAD, ctypes.byref(s), 128, 6) == 0    # 2 M tiles, 8 epilogue warps
    assert L.convgemm_tune_set(tc.TUNE_FWD_FP8, ctypes.byref(s), 128, 1) == 1
    assert L.convgemm_tune_set(tc.TUNE_WGRAD, ctypes.byref(s), 0, 3) == 0
    assert L.convgemm_tune_set(tc.TUNE_WGRAD, ctypes.byref(s), 256, 3 | tc.WGRAD_X_ON_A | tc.WGRAD_IM2COL_X) == 0
    assert L.convgemm_tune_set(tc.TUNE_WGRAD, ctypes.byref(s), 256, 0x40000) == 1   # no such flag
    tc.tune_clear()


def test_set_pdl_is_per_thread_and_restores_default(cglib, monkeypatch):
    """convgemm_set_pdl switches programmatic launches for the calling thread and
    returns the previous setting; -1 goes back to the environment's default."""
    import threading
    default = 0 if os.environ.get("CONVGEMM_NO_PDL") == "1" else 1
    assert cglib.set_pdl(0) == default
    seen = []
    t = threading.Thread(target=lambda: seen.append(cglib.set_pdl(-1)))
    t.start()
    t.join()
    assert seen == [default]              # another thread still has the default
    assert cglib.set_pdl(1) == 0
    assert cglib.set_pdl(-1) == 1
    assert cglib.set_pdl(-1) == default


def test_batch_norm_training_entry_points_validate_without_gpu(cglib):
    """Workspace sizes of the statistics forward and argument checks of the fold / apply."""
    L = cglib.lib()
    s = cglib.Shape.of(2, 14, 14, 64, 128, 3, 3, 1, 1)
    groups = -(-(2 * 14 * 14) // 32)
    chunks = -(-groups // 256)
    assert L.convgemm_fwd_bf16_stats_workspace_size(ctypes.byref(s)) == chunks * 2 * 128 * 8 + groups * 2 * 128 * 4
    stem = cglib.Shape.of(2, 20, 20, 3, 64, 7, 7, 3, 3, 2, 2)       # small-channel kernel: 4 groups per row chunk
    assert L.convgemm_fwd_bf16_stats_workspace_size(ctypes.byref(stem)) == 1 * 2 * 64 * 8 + 2 * 10 * 4 * 2 * 64 * 4
    bad = cglib.Shape.of(0, 14, 14, 64, 128, 3, 3, 1, 1)
    assert L.convgemm_fwd_bf16_stats_workspace_size(ctypes.byref(bad)) == 0
    assert L.convgemm_fwd_bf16_stats(ctypes.byref(s), None, None, None, None, None, 0, None, None, 0, None) == 1
    assert L.convgemm_fwd_bf16_stats(ctypes.byref(s), 16, 16, 16, None, None, 0, 16, 16, 8, None) != 0   # workspace
    assert "workspace" in cglib.last_error()[1]
    assert L.convgemm_bn_stats_fold(0, 16, 10, None, None, 1e-5, 16, 16, None, None, None) == 1
    assert L.convgemm_bn_stats_fold(8, 16, 0, None, None, 1e-5, 16, 16, None, None, None) == 1
    assert L.convgemm_bn_apply_bf16(10, 12, 16, 16, 16, 1, 16, None) == 1     # kn % 8


def test_stem_weight_gradient_plan_without_gpu(cglib):
    """Weight-gradient planning needs no GPU. The ResNet-50 stem (c <= 8, stride 2, kn = 64) plans
    one FP32 partial per CTA of its slab kernel (bands of 8 output rows, one CTA per SM), whatever
    tile configuration is set. The workspace holds those partials plus the fixed-order reduction's
    group sums (about eight partials per group once there are more than 16)."""
    from convgemm_gb300 import tc
    import torch
    cg = cglib
    s = cg.Shape.of(64, 224, 224, 3, 64, 7, 7, 3, 3, 2, 2)
    sms = torch.cuda.get_device_properties(0).multi_processor_count if torch.cuda.is_available() else 148
    splits = min(sms, 64 * 14)
    g = min(splits // 8, 32)
    per = -(-splits // g)
    groups = -(-splits // per)
    try:
        for bn, aux in ((0, 0), (128, 7), (64, 3 | tc.WGRAD_X_ON_A)):
            if bn or aux:
                tc.tune_set(tc.TUNE_WGRAD, s, bn, aux)
            assert tc.wgrad_bf16_plan(s)[:2] == (64, splits)
            assert tc.wgrad_bf16_workspace_size(s) == 4 * (splits + groups) * (49 * 8) * 64
        # stride 1 (VGG's first layer) stays on the general kernel: its own split heuristic
        v = cg.Shape.of(32, 224, 224, 3, 64, 3, 3, 1, 1, 1, 1)
        tc.tune_set(tc.TUNE_WGRAD, v, 64, 5)
        assert tc.wgrad_bf16_plan(v)[:2] == (64, 5)
    finally:
        tc.tune_clear()


def test_weight_gradient_flags_in_plan_without_gpu(cglib):
    """The weight-gradient aux flags are parsed off the split count: X on the A side takes N tiles
    of 64 / 128 / 256 output channels, and the split count in bits 0-15 still applies."""
    from convgemm_gb300 import tc
    cg = cglib
    s = cg.Shape.of(8, 14, 14, 256, 256, 3, 3, 1, 1, 1, 1)
    try:
        for bn, splits in ((128, 4), (256, 2), (64, 7)):
            tc.tune_set(tc.TUNE_WGRAD, s, bn, splits | tc.WGRAD_X_ON_A)
            assert tc.wgrad_bf16_plan(s)[:2] == (bn, splits)
        tc.tune_set(tc.TUNE_WGRAD, s, 256, 3 | tc.WGRAD_IM2COL_X)
        assert tc.wgrad_bf16_plan(s)[:2] == (256, 3)
    finally:
        tc.tune_clear()


def test_shipped_tuning_table_entries_parse():
    """Every tuned forward / input-gradient / weight-gradient entry of the shipped GB300 table
    names its tile width, aux flags, kernel, ring stages and cluster size, within the ranges the
    library accepts (convgemm_tune_set / convgemm_tune_describe)."""
    import json
    path = os.path.join(ROOT, "convgemm_gb300", "autotune_gb300.json")
    table = json.load(open(path))["NVIDIA GB300"]
    ops = [k for k in table if "|" in k and k.split("|")[0].split(".")[0] in ("fwd", "dgrad", "wgrad")]
    assert len(ops) >= 100
    for k in ops:
        e = table[k]
        op = k.split(".")[0]
        assert e["bn"] in (0, 64, 128, 256), k
        aux = int(e["splits"])
        if op == "wgrad":
            assert aux >= 0 and (aux & ~0x3FBFFFF) == 0, k
        else:
            assert (aux & ~24) in (0, 1, 2, 5, 6), k
        assert e["kernel"] in (0, 1, 2), k
        assert e["stages"] in (0, 2, 3, 4, 6, 8), k
        assert 1 <= e["cluster"] <= 8, k
        if e["kernel"] == 0:
            assert e["stages"] >= 2, k
        shape = [int(v) for v in k.split("|")[1].split("x")]
        assert len(shape) == 13 and min(shape[:7]) >= 1, k
