"""The Python layer rejects tensors and arrays the kernels cannot take (host
memory, wrong type, not contiguous, too short) before any library call: the
C ABI gets plain pointers and could not tell.  Wrapper objects are built
without a GPU and the library loader is replaced by one that fails."""
import numpy as np
import pytest
import torch

import fastload_gb300 as fl
from fastload_gb300 import batch as batch_mod
from fastload_gb300 import compare
from fastload_gb300 import plan as plan_mod


@pytest.fixture
def no_library(monkeypatch):
    def called(*a, **k):
        raise AssertionError("the library was called")

    for mod in (plan_mod, batch_mod, compare):
        monkeypatch.setattr(mod, "load", called)


def fake_plan(m=6, n=5, forms=None):
    p = fl.Plan.__new__(fl.Plan)
    p._h, p._keep, p.m, p.n = None, None, m, n
    p._form_kinds = dict(forms or {})
    return p


def rejects(fn):
    with pytest.raises(fl.FastLoadArgumentError) as e:
        fn()
    assert isinstance(e.value, fl.FastLoadError) and isinstance(e.value, ValueError) and e.value.code == -1
    return str(e.value)


def test_spmv_needs_device_tensors(no_library):
    p = fake_plan()
    assert "CUDA tensor" in rejects(lambda: p.spmv(torch.zeros(5, dtype=torch.float64)))
    assert "CUDA tensor" in rejects(lambda: p.spmv(np.zeros(5)))
    assert "CUDA tensor" in rejects(lambda: p.permute_x(np.zeros(5), out=torch.zeros(5, dtype=torch.float64)))


def test_spmv_host_checks_length_type_and_layout(no_library):
    p = fake_plan()
    assert "at least 5" in rejects(lambda: p.spmv_host(np.zeros(4)))
    assert "float64" in rejects(lambda: p.spmv_host(np.zeros(5), y=np.zeros(6, np.float32)))
    assert "at least 6" in rejects(lambda: p.spmv_host(np.zeros(5), y=np.zeros(5)))
    strided = np.zeros((6, 2))[:, 0]
    assert "C-contiguous" in rejects(lambda: p.spmv_host(np.zeros(5), y=strided))
    assert "C-contiguous" in rejects(lambda: p.spmv_host_async(np.zeros(5), strided))
    assert "at least 5" in rejects(lambda: p.spmv_host_async(np.zeros(3), np.zeros(6)))
    assert "float64" in rejects(lambda: p.spmv_host_async(np.zeros(5, np.float32), np.zeros(6)))


def test_spmv_form_follows_the_form(no_library):
    p = fake_plan(forms={0: (fl.VALUES_F32, False), 1: (fl.VALUES_F64, True)})
    assert "FP64 y" in rejects(lambda: p.spmv_form(0, None, y_f32=True))
    assert "FP32 y" in rejects(lambda: p.spmv_form(1, None, y_f32=False))
    assert "float32" in rejects(lambda: p.spmv_form(0, torch.zeros(5, dtype=torch.float32)))
    assert "float64" in rejects(lambda: p.spmv_form(1, np.zeros(5)))


def test_batch_and_comparators(no_library):
    b = batch_mod.Batch.__new__(batch_mod.Batch)
    b._h, b.value_type, b.y_f32, b.m, b.n = None, fl.VALUES_F32, True, 6, 5
    assert "float32" in rejects(lambda: b.spmv(torch.zeros(5, dtype=torch.float32)))
    assert "float32" in rejects(lambda: b.spmv_graph(torch.zeros(5, dtype=torch.float64)))
    cs = compare.CuSparse.__new__(compare.CuSparse)
    cs._h, cs.m, cs.n = None, 6, 5
    assert "CUDA tensor" in rejects(lambda: cs.spmv(torch.zeros(5, dtype=torch.float64)))
    cp = torch.zeros(6, dtype=torch.int32)
    assert "CUDA tensor" in rejects(lambda: compare.csc_spmv_naive(6, cp, cp, cp, torch.zeros(5)))


def test_fastload_spmv_checks_the_slide_matrix(monkeypatch):
    from fastload_gb300 import host

    monkeypatch.setattr(host, "load", lambda: (_ for _ in ()).throw(AssertionError("the library was called")))
    z = np.zeros
    sm = host.SlideMatrix(sortval=z(3), sortrowidx=z(3, np.int32), tile_ptr=z(2, np.int32), tile_len=z(2, np.int32),
                          tile_colidx=z(2, np.int32), tile_tall=z(2, np.int32), tile_format=z(2, np.int32),
                          countrow=z(3, np.int32), segmentoffset=z(1, np.int32), sortrowindex=z(3, np.int32),
                          tilenum=2, segsum=0)
    assert "tile_ptr (2 < 3)" in rejects(lambda: host.FastLoad_spmv(sm, 3, 2, 4, z(2)))
    sm.tile_ptr = z(3, np.int32)
    assert "sortval (3 < 5)" in rejects(lambda: host.FastLoad_spmv(sm, 5, 2, 4, z(2)))
    assert "y_golden" in rejects(lambda: host.FastLoad_spmv(sm, 3, 2, 4, z(2), y_golden=z(3)))


def test_tuner_network_checks_shapes(monkeypatch):
    from fastload_gb300 import tuner

    net = tuner.Network.__new__(tuner.Network)
    net._h, net.shape = None, (24, 64, 64, 6)
    monkeypatch.setattr(tuner, "load", lambda: (_ for _ in ()).throw(AssertionError("the library was called")))
    assert "expected (rows, 24)" in rejects(lambda: net.forward_raw(np.zeros((3, 23))))
    assert "expected (rows, 24)" in rejects(lambda: net.forward_raw(np.zeros(24)))
    assert "expected (3, 6)" in rejects(lambda: net.grad_raw(np.zeros((3, 24)), np.zeros((2, 6))))
    assert "expected (3, 6)" in rejects(lambda: net.grad_raw(np.zeros((3, 24)), np.zeros((3, 6)), np.zeros((3, 5))))
    assert "expected (4, 6)" in rejects(lambda: net.fit(np.zeros((4, 24)), np.ones((4, 5)), epochs=1))
    monkeypatch.setattr(tuner.Network, "num_params", property(lambda self: 10))
    assert "9 values" in rejects(lambda: net.set_params(np.zeros(9)))


def test_plan_create_rejects_negative_sizes(no_library):
    assert "negative size" in rejects(lambda: fl.Plan.from_csr(-1, 3, np.zeros(1), np.zeros(0), np.zeros(0)))
