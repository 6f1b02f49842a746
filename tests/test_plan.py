"""Plans and the schedule tuner (mdg_plan_*, mdg_tune_cache_*): the JSON
cache round trip and argument checks on the CPU; on the GPU, tuning keeps
the bits of mdg_gemm and seeds later plans of the same shape class."""
import ctypes
import json

import numpy as np
import pytest

from conftest import pkg

CACHE = {"NVIDIA GB300|13000": {"2 4 28 28 1024 1024 1024": {"engine": 2, "parts": 2,
                                                            "raster": 8, "pace": 128,
                                                            "ms": 1.25},
                                "2 2 14 14 256 256 64": {"engine": 1, "parts": 0,
                                                        "raster": 0, "pace": -1, "ms": 0.01},
                                "batch 256 0123456789abcdef": {"tiles": 2, "ms": 13.5},
                                "batch 7 fedcba9876543210": {"tiles": 3, "split": 0,
                                                             "ms": 0.5}},
         "other|1": {}}


def test_tune_cache_json_round_trip(tmp_path):
    api = pkg("api")
    api.tune_cache_clear()
    src = tmp_path / "in.json"
    src.write_text(json.dumps(CACHE))
    api.tune_cache_load(src)
    assert api.tune_cache_size() == 4
    out = tmp_path / "out.json"
    api.tune_cache_save(out)
    back = json.loads(out.read_text())
    assert back["NVIDIA GB300|13000"] == CACHE["NVIDIA GB300|13000"]
    api.tune_cache_load(out)  # merging the same entries again changes nothing
    assert api.tune_cache_size() == 4
    api.tune_cache_clear()
    assert api.tune_cache_size() == 0


def test_tune_cache_rejects_bad_files(tmp_path):
    L = pkg("_lib").lib()
    bad = tmp_path / "bad.json"
    for text in ("{", "[]", '{"a": {"b": {"engine": "x"}}}', '{"a": 1}', '{"a": {}} trailing'):
        bad.write_text(text)
        assert L.mdg_tune_cache_load(str(bad).encode()) == 4, text
    # schedule values outside what mdg_gemm accepts reject the whole file
    for field, value in (("engine", "1e300"), ("engine", "-1"), ("engine", "4"),
                         ("engine", "nan"), ("parts", "9"), ("parts", "1.5"),
                         ("raster", "-1"), ("raster", "inf"), ("raster", "2e6"),
                         ("tiles", "4"), ("tiles", "-1"), ("pace", "-2"), ("pace", "70000"),
                         ("split", "2"), ("split", "-1"),
                         ("ms", "-1"), ("ms", "nan")):
        bad.write_text('{"d": {"ok": {"engine": 2, "parts": 1}, '
                       f'"s": {{"{field}": {value}}}}}}}')
        assert L.mdg_tune_cache_load(str(bad).encode()) == 4, (field, value)
    assert L.mdg_tune_cache_load(str(tmp_path / "missing.json").encode()) == 7
    assert L.mdg_tune_cache_load(None) == 3
    assert L.mdg_tune_cache_size() == 0


def test_plan_arguments_without_gpu():
    L = pkg("_lib").lib()
    h = ctypes.c_void_p()
    assert L.mdg_plan_create(0, 3, 4, 4, 4, None, ctypes.byref(h)) == 1
    assert L.mdg_plan_create(7, 4, 4, 4, 4, None, ctypes.byref(h)) == 4
    assert L.mdg_plan_create(2, 4, -1, 4, 4, None, ctypes.byref(h)) == 2
    assert L.mdg_plan_create(2, 4, 4, 4, 4, None, None) == 3
    assert L.mdg_plan_run(None, None, 1, None, 1, None, 1, None) == 3
    assert L.mdg_plan_workspace_bytes(None) == 0
    L.mdg_plan_destroy(None)


@pytest.mark.gpu
def test_tuned_plan_keeps_bits_and_seeds_later_plans(inputs, tmp_path):
    import torch
    api = pkg("api")
    api.tune_cache_clear()
    P, A, B = inputs.workload("qd1024", 1024, 768, 512)
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    ref = api.gemm(dA, dB, "slice_bf16").cpu().numpy()
    plan = api.Plan("slice_bf16", P, 1024, 768, 512)
    assert plan.schedule()["engine"] == 0  # nothing cached yet: automatic
    C = torch.empty((1024, 768, P), dtype=torch.float64, device="cuda")
    plan.tune(dA, dB, C)
    assert np.array_equal(C.cpu().numpy(), ref)
    chosen = plan.schedule()
    assert chosen["engine"] in (1, 2) and api.tune_cache_size() == 1
    assert np.array_equal(plan.run(dA, dB).cpu().numpy(), ref)
    again = api.Plan("slice_bf16", P, 1000, 700, 500)  # same padded shape class
    assert again.schedule() == chosen
    assert np.array_equal(again.run(dA[:1000, :500].contiguous(), dB[:500, :700].contiguous())
                          .cpu().numpy(), api.gemm(dA[:1000, :500].contiguous(),
                                                   dB[:500, :700].contiguous(),
                                                   "slice_bf16").cpu().numpy())
    path = tmp_path / "tune.json"
    api.tune_cache_save(path)
    api.tune_cache_clear()
    api.tune_cache_load(path)
    assert api.Plan("slice_bf16", P, 1024, 768, 512).schedule() == chosen
    plain = api.Plan("plain", P, 64, 64, 64)
    plain.tune(dA[:64, :64].contiguous(), dB[:64, :64].contiguous(),
               torch.empty((64, 64, P), dtype=torch.float64, device="cuda"))
    assert api.tune_cache_size() == 1  # nothing to tune for the plain form
    for p_ in (plan, again, plain):
        p_.close()
    api.tune_cache_clear()
