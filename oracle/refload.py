"""Import the unmodified reference TensorOrder (test infrastructure only).

The reference's pure-Python modules are imported from its own ``src/``
directory; its five Cython extension modules come from ``oracle/_ref/lib``
(built by ``oracle/build_ref.py``).  A ``sys.meta_path`` finder maps exactly
those five dotted names to the compiled files, so nothing is copied out of, or
written into, the reference checkout.

Two environment shims are applied, both needed because the reference pins
numpy 1.18 (``requirements.txt:37``):

* ``numpy.object = object`` -- ``numpy_apis.py:21`` uses the alias removed in
  numpy 1.24.
"""
import glob
import importlib.abc
import importlib.machinery
import importlib.util
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")

_EXTENSIONS = (
    "tensor_network.tensor_network",
    "contraction_methods.contraction_tree",
    "contraction_methods.factor_tree_method",
    "decompositions.tree_decomposition",
    "decompositions.branch_decomposition",
)


def reference_src():
    """``src/`` of the reference checkout: ``TOGB_REFERENCE_ROOT``, else
    ``../reference`` next to this repository."""
    default = os.path.join(os.path.dirname(HERE), os.pardir, "reference")
    return os.path.join(os.path.normpath(os.environ.get("TOGB_REFERENCE_ROOT", default)), "src")


def available():
    """True when both the reference checkout and the built extensions exist."""
    return os.path.isdir(reference_src()) and os.path.exists(os.path.join(REF_OUT, "lib", ".built"))


class _ExtensionFinder(importlib.abc.MetaPathFinder):
    def find_spec(self, fullname, path, target=None):
        if fullname not in _EXTENSIONS:
            return None
        pkg, mod = fullname.split(".")
        hits = glob.glob(os.path.join(REF_OUT, "lib", pkg, mod + ".*.so"))
        if not hits:
            raise ImportError("reference extension %s is not built (run oracle/build_ref.py)" % fullname)
        loader = importlib.machinery.ExtensionFileLoader(fullname, hits[0])
        return importlib.util.spec_from_file_location(fullname, hits[0], loader=loader)


_loaded = None


def load():
    """Import the reference and return a namespace of the modules used by tests."""
    global _loaded
    if _loaded is not None:
        return _loaded
    if not available():
        raise RuntimeError("reference oracle unavailable: build it with oracle/build_ref.py")
    import numpy

    if not hasattr(numpy, "object"):
        numpy.object = object
    sys.setrecursionlimit(100000)
    if not any(isinstance(f, _ExtensionFinder) for f in sys.meta_path):
        sys.meta_path.insert(0, _ExtensionFinder())
    src = reference_src()
    if src not in sys.path:
        sys.path.insert(0, src)
    import types

    import contraction_methods
    import tensor_network
    import util
    from tensor_network import sliced_execution_plan
    from tensor_network.tensor_apis import base_api, numpy_apis
    import planning
    import execution

    _loaded = types.SimpleNamespace(
        tensor_network=tensor_network,
        contraction_methods=contraction_methods,
        util=util,
        sliced_execution_plan=sliced_execution_plan,
        base_api=base_api,
        numpy_apis=numpy_apis,
        planning=planning,
        execution=execution,
    )
    return _loaded


class _cwd:
    def __init__(self, path):
        self.path = path

    def __enter__(self):
        self.old = os.getcwd()
        os.chdir(self.path)

    def __exit__(self, *exc):
        os.chdir(self.old)


def plan_cnf(cnf_text, weights="unweighted", planner="line-Flow", seed=0, timeout=10.0,
             minimum_slice=0, rank_limit=30, slicer="greedy_mem"):
    """Run the reference's Reduction + Planning + Slicing stages on DIMACS text.

    Follows ``tensororder.py:386-270``: ``cnf_count`` (reduction), ``planning.run``
    (anytime planner under a ``TimeoutTimer``), then
    ``slicer.slice_until(plan, memory=None, rank=rank_limit, slices=minimum_slice)``.
    Returns the reference ``SlicedExecutionPlan``.
    """
    import io
    import random

    ref = load()
    random.seed(seed)
    weight_format = ref.util.WeightFormat[weights]
    network = ref.tensor_network.ALL_CONSTRUCTIONS["wmc"](io.StringIO(cnf_text), weight_format)
    solver = ref.contraction_methods.ALL_SOLVERS[planner]
    with _cwd(REF_OUT):
        with ref.util.TimeoutTimer(timeout) as timer:
            plan, _ = ref.planning.run(solver, network, seed, timer, None, rank_limit=None,
                                       performance_factor=None, mem_limit=None, slicer=None)
    if plan is None:
        raise RuntimeError("reference planner produced no plan")
    ref.tensor_network.ALL_SLICERS[slicer].slice_until(plan, memory=None, rank=rank_limit,
                                                      slices=minimum_slice)
    return plan


def reference_count(plan, entry_type="float64", num_slice_limit=None, thread_limit=None):
    """Contract a reference plan with the reference's own numpy backend
    (``numpy_apis.py:4-70`` via ``base_api.py:17-28``)."""
    ref = load()
    api = ref.tensor_network.ALL_APIS["numpy"]()
    api.add_argument("entry_type", entry_type)
    if thread_limit is not None:
        api.add_argument("thread_limit", thread_limit)
    return api.contract_sliced(plan, num_slice_limit=num_slice_limit)
