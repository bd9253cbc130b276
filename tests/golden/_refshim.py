"""Import the reference package with stand-ins for its absent third-party modules.

This module is used only by ``make_golden.py`` to run the reference's own
JAX backend (``pespace/detector/_jax_impl/*``, ``pespace/inference/likelihood_jax.py``)
with NumPy standing in for ``jax.numpy``.  The taichi, h5py and ripplegw modules
are replaced by permissive stubs so that the reference modules import; none of
their taichi kernels is ever executed.  Every array the golden fixtures hold is
therefore computed by the reference's own source lines.
"""

import sys
import types

import numpy as np


class _Anything:
    """Object that accepts any attribute access, call or decoration."""

    def __init__(self, name="stub"):
        self._name = name

    def __getattr__(self, item):
        return _Anything(f"{self._name}.{item}")

    def __call__(self, *args, **kwargs):
        # used as a decorator: return the decorated object unchanged
        if len(args) == 1 and not kwargs and (callable(args[0]) or isinstance(args[0], type)):
            return args[0]
        return _Anything(f"{self._name}()")

    def __iter__(self):
        return iter(())

    def __repr__(self):
        return f"<stub {self._name}>"


def _make_taichi():
    ti = types.ModuleType("taichi")
    identity = lambda obj=None, *a, **k: obj  # noqa: E731
    ti.kernel = identity
    ti.func = identity
    ti.data_oriented = identity
    ti.static = lambda x, *a: x
    ti.template = lambda *a, **k: None
    ti.types = _Anything("taichi.types")
    ti.Struct = _Anything("taichi.Struct")
    ti.StructField = type("StructField", (), {})
    ti.Field = type("Field", (), {})
    ti.Vector = _Anything("taichi.Vector")
    ti.field = _Anything("taichi.field")
    ti.f64 = "f64"
    ti.f32 = "f32"
    ti.u32 = int
    ti.u8 = int
    ti.i32 = int

    class _FP:
        def to_string(self):
            return "f64"

    class _Cfg:
        default_fp = _FP()

    ti.lang = types.SimpleNamespace(impl=types.SimpleNamespace(current_cfg=lambda: _Cfg()))
    tm = types.ModuleType("taichi.math")
    tm.__getattr__ = lambda name: _Anything(f"taichi.math.{name}")
    ti.math = tm
    ti.__getattr__ = lambda name: _Anything(f"taichi.{name}")
    return ti, tm


def _make_jax():
    jax = types.ModuleType("jax")
    jax.numpy = np
    jax.config = types.SimpleNamespace(jax_enable_x64=True)

    def tree_map(fn, tree):
        if isinstance(tree, dict):
            return {k: tree_map(fn, v) for k, v in tree.items()}
        if isinstance(tree, tuple) and hasattr(tree, "_fields"):
            return type(tree)(*[tree_map(fn, v) for v in tree])
        if isinstance(tree, (list, tuple)):
            return type(tree)(tree_map(fn, v) for v in tree)
        return fn(tree)

    jax.tree = types.SimpleNamespace(map=tree_map)
    jax.tree_util = types.SimpleNamespace(register_pytree_node_class=lambda cls: cls)
    jax.lax = types.SimpleNamespace(optimization_barrier=lambda x: x)
    return jax


def install(reference_root):
    """Install the stubs and put ``reference_root`` on ``sys.path``."""
    ti, tm = _make_taichi()
    sys.modules["taichi"] = ti
    sys.modules["taichi.math"] = tm
    jax = _make_jax()
    sys.modules["jax"] = jax
    sys.modules["jax.numpy"] = np
    sys.modules["h5py"] = types.ModuleType("h5py")
    rip = types.ModuleType("ripplegw")
    rip_w = types.ModuleType("ripplegw.waveforms")
    rip_xas = types.ModuleType("ripplegw.waveforms.IMRPhenomXAS")
    rip_xas.gen_IMRPhenomXAS_hphctf = None
    rip_xhm = types.ModuleType("ripplegw.waveforms.IMRPhenomXHM")
    rip_xhm.gen_IMRPhenomXHM_hphctf_modes = None
    sys.modules.update(
        {
            "ripplegw": rip,
            "ripplegw.waveforms": rip_w,
            "ripplegw.waveforms.IMRPhenomXAS": rip_xas,
            "ripplegw.waveforms.IMRPhenomXHM": rip_xhm,
        }
    )
    if reference_root not in sys.path:
        sys.path.insert(0, reference_root)
