"""
With xarray importable, importing harmonica_gb300 registers the layer
accessors on ``xarray.Dataset`` (``.prism_layer`` and ``.tesseroid_layer``,
as harmonica does at prisms/layer.py:157 and tesseroid_layer.py:183), and
``prism_layer`` / ``tesseroid_layer`` return Datasets on which they work.

xarray is not installed in this environment, so a child process puts a small
stand-in module named ``xarray`` on ``sys.modules`` before the import: a
``Dataset`` with coordinates, data variables and ``attrs``, and
``register_dataset_accessor`` doing what xarray's does (a cached property per
dataset).  When the real xarray is importable the same checks also run on it.
"""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_FAKE_XARRAY = r'''
import sys, types
import numpy as np

class DataArray:
    def __init__(self, values):
        self.values = np.asarray(values)
    @property
    def size(self):
        return self.values.size

class _Coords(dict):
    def __setitem__(self, key, value):
        values = value[1] if isinstance(value, tuple) else value
        super().__setitem__(key, DataArray(values))

class Dataset:
    def __init__(self, data_vars=None, coords=None):
        self.coords = _Coords()
        self.data_vars = {k: DataArray(v[1]) for k, v in (data_vars or {}).items()}
        self.attrs = {}
        for k, v in (coords or {}).items():
            self.coords[k] = v
    def __getattr__(self, name):
        for table in ("coords", "data_vars"):
            entries = self.__dict__.get(table, {})
            if name in entries:
                return entries[name]
        raise AttributeError(name)
    def __getitem__(self, name):
        return self.data_vars[name] if name in self.data_vars else self.coords[name]

registered = {}

def register_dataset_accessor(name):
    def decorator(cls):
        registered[name] = cls
        cache = "_accessor_" + name
        def get(self):
            if cache not in self.__dict__:
                self.__dict__[cache] = cls(self)
            return self.__dict__[cache]
        setattr(Dataset, name, property(get))
        return cls
    return decorator

xr = types.ModuleType("xarray")
Dataset.__module__ = DataArray.__module__ = "xarray"
xr.Dataset, xr.DataArray = Dataset, DataArray
xr.register_dataset_accessor, xr.registered = register_dataset_accessor, registered
sys.modules["xarray"] = xr
'''

_CHECKS = r'''
import json
import numpy as np
try:
    import xarray as xr
except ImportError:
    xr = None
import harmonica_gb300 as hg

report = {}
if hasattr(xr, "registered"):
    report["registered"] = {k: v.__name__ for k, v in xr.registered.items()}
easting = np.linspace(0, 900, 10)
northing = np.linspace(50, 450, 5)
surface = np.arange(50.0).reshape(5, 10)
layer = hg.prism_layer((easting, northing), surface, 10.0,
                       properties={"density": np.full((5, 10), 2670.0)})
report["prism_type"] = type(layer).__module__ + "." + type(layer).__name__
acc = layer.prism_layer
report["prism_accessor"] = type(acc).__name__
report["spacing"] = [float(v) for v in acc.spacing]
report["boundaries"] = [float(v) for v in acc.boundaries]
report["shape"] = list(acc.shape)
report["n_prisms"] = int(acc._to_prisms().shape[0])
report["prism_11"] = [float(v) for v in acc.get_prism((1, 1))]
lon = np.linspace(-10, 10, 11)
lat = np.linspace(-5, 5, 6)
tl = hg.tesseroid_layer((lon, lat), np.full((6, 11), 6.372e6), 6.371e6,
                        properties={"density": np.ones((6, 11))})
report["tesseroid_accessor"] = type(tl.tesseroid_layer).__name__
report["tesseroid_shape"] = list(tl.tesseroid_layer.shape)
print(json.dumps(report))
'''


def _run(prelude):
    code = prelude + "\nimport sys\nsys.path.insert(0, %r)\n" % ROOT + _CHECKS
    run = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                         timeout=300)
    assert run.returncode == 0, run.stderr[-3000:]
    return json.loads(run.stdout.strip().splitlines()[-1])


def _check(report):
    assert report["prism_accessor"] == "DatasetAccessorPrismLayer"
    assert report["spacing"] == [100.0, 100.0]
    assert report["boundaries"] == [-50.0, 950.0, 0.0, 500.0]
    assert report["shape"] == [5, 10]
    assert report["n_prisms"] == 50
    # (northing index 1, easting index 1): centre (100, 150), surface 11 over 10
    assert report["prism_11"] == [50.0, 150.0, 100.0, 200.0, 10.0, 11.0]
    assert report["tesseroid_accessor"] == "DatasetAccessorTesseroidLayer"
    assert report["tesseroid_shape"] == [6, 11]


def test_accessors_registered_on_xarray_datasets():
    report = _run(_FAKE_XARRAY)
    assert report["registered"] == {"prism_layer": "DatasetAccessorPrismLayer",
                                    "tesseroid_layer": "DatasetAccessorTesseroidLayer"}
    assert report["prism_type"] == "xarray.Dataset"
    _check(report)


def test_accessors_on_real_xarray_when_installed():
    """Runs the same checks on the real xarray where it is installed; without
    it, on the numpy stand-in containers."""
    try:
        import xarray  # noqa: F401
    except ImportError:
        report = _run("")
        assert report["prism_type"] == "harmonica_gb300.layer.PrismLayer"
    else:
        report = _run("")
        assert report["prism_type"].startswith("xarray.")
    _check(report)
