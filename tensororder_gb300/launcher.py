"""Run the reference's own CLI with the GB300 plugins registered.

    python -m tensororder_gb300.launcher --reference-src PATH/TO/TensorOrder/src \\
        tensororder [tensororder.py options] --tensor_library gb300-split < formula.cnf
    python -m tensororder_gb300.launcher --reference-src ... execution [execution.py options] plan.con

The reference resolves ``--tensor_library`` through ``util.TaggedChoice`` over
the live ``tensor_network.ALL_APIS`` dict (``util.py:249-252``), so adding the
plugins before the click command runs is the whole integration; no reference
file is edited.  ``numpy.object`` is restored because ``numpy_apis.py:21``
still names that alias, which numpy 1.24 removed.
"""
import argparse
import os
import sys


def main(argv=None):
    ap = argparse.ArgumentParser(add_help=False)
    ap.add_argument("--reference-src", required=True)
    ap.add_argument("entry", choices=["tensororder", "execution", "planning"])
    args, rest = ap.parse_known_args(argv)
    import numpy

    if not hasattr(numpy, "object"):
        numpy.object = object
    # util.FileLocator resolves solver binaries relative to the working
    # directory (util.py:288-297), so run from the reference's src/ as usual.
    sys.path.insert(0, os.path.abspath(args.reference_src))
    from tensororder_gb300 import api

    api.register()
    module = __import__(args.entry)
    command = {"tensororder": "run", "execution": "measure", "planning": "measure"}[args.entry]
    getattr(module, command)(args=rest, prog_name=args.entry)


if __name__ == "__main__":
    main()
