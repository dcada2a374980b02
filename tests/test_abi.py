"""The C ABI library on CPU: it loads, exports every declared entry point,
validates arguments, and its host-only generators are deterministic."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import krabmaga_gb300 as kg
from krabmaga_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(kb_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    syms = declared_symbols()
    assert len(syms) >= 30
    lib = C.CDLL(L.LIB_PATH)
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_version_and_error_string():
    assert b"sm_103a" in L.lib.kb_version()
    assert isinstance(L.last_error(), str)


def test_null_arguments_are_rejected():
    assert L.lib.kb_field_create(None, None) == L.KB_ERR_ARG
    assert "null" in L.last_error()
    assert L.lib.kb_field_set_locations(None, 0, None, None, None) == L.KB_ERR_ARG


def test_bad_geometry_is_rejected():
    desc = L.FieldDesc(0.0, 10.0, 0.5, 1, 0, 0)
    h = C.c_void_p()
    assert L.lib.kb_field_create(C.byref(desc), C.byref(h)) == L.KB_ERR_ARG
    desc = L.FieldDesc(10.0, 10.0, float("nan"), 1, 0, 0)
    assert L.lib.kb_field_create(C.byref(desc), C.byref(h)) == L.KB_ERR_ARG


@pytest.mark.skipif(kg.device_count() > 0, reason="checks the no-device path")
def test_no_device_fails_loudly():
    desc = L.FieldDesc(10.0, 10.0, 0.5, 1, 0, 0)
    h = C.c_void_p()
    assert L.lib.kb_field_create(C.byref(desc), C.byref(h)) == L.KB_ERR_NO_DEVICE
    with pytest.raises(L.KbError):
        kg.Field2D(10.0, 10.0, 0.5, True)


def test_uniform_generator_is_deterministic_and_in_range():
    a = kg.gen_uniform(5000, 6476.3447, 6476.3447, 7, 1.0)
    b = kg.gen_uniform(5000, 6476.3447, 6476.3447, 7, 1.0)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    ids, xy, dxy = a
    assert np.array_equal(ids, np.arange(5000))
    assert (xy >= 0).all() and (xy <= np.float32(6476.3447)).all()
    norms = np.sqrt((dxy.astype(np.float64) ** 2).sum(1))
    assert np.allclose(norms, 1.0, atol=1e-6)
    ang = np.arctan2(dxy[:, 1], dxy[:, 0])
    hist, _ = np.histogram(ang, bins=8, range=(-np.pi, np.pi))
    assert hist.min() > 500  # uniform in angle
    c = kg.gen_uniform(10, 100.0, 100.0, 8, 0.0)
    assert (c[2] == 0).all()  # the reference's last_d = (0, 0) initial heading


def test_clustered_generator_shape():
    ids, xy, dxy = kg.gen_clustered(4096, 12952.0, 12952.0, 256, 40.0, 0.3, 11)
    assert (xy >= 0).all() and (xy < 12952.0).all()
    # boids of one cluster sit within a few sigma of each other (on the torus)
    c0 = xy[ids % 256 == 0]
    d = np.abs(c0 - c0[0])
    d = np.minimum(d, 12952.0 - d)
    assert np.percentile(np.sqrt((d ** 2).sum(1)), 90) < 6 * 40.0


def test_field_mirror_api_names():
    # the Python mirror keeps the reference's Field2D method names
    for name in ["set_object_location", "remove_object_location", "lazy_update",
                 "get_neighbors_within_relax_distance", "get_neighbors_within_distance",
                 "get_objects", "get_objects_unbuffered", "num_objects_at_location",
                 "get_empty_bags", "get_random_empty_bag", "iter_objects",
                 "iter_objects_unbuffered"]:
        assert callable(getattr(kg.Field2D, name))
