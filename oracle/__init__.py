"""CPU oracle for the TensorOrder contraction path -- test infrastructure.

``contract.py`` restates the reference's numpy FP64 execution of a sliced plan;
``build_ref.py`` and ``refload.py`` build and import the unmodified reference
(where its checkout is present) to pin that restatement.  Product code never
imports this package; only tests, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` do.
"""
