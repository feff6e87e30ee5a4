"""Run torchmorph's own test suite against this package (a drop-in check).

Usage::

    python tests/run_reference_suite.py --reference PATH [--mode api|boundary] [pytest args]

PATH is a torchmorph checkout (its ``test/`` folder and, for ``--mode boundary``,
its ``torchmorph/`` Python package).  The suite needs a CUDA device; it runs in a
temporary folder with a ``conftest.py`` that installs one of two shims:

* ``api`` (default): ``import torchmorph`` resolves to ``torchmorph_gb300`` and
  its submodules, so every public operator the tests call is this package's;
* ``boundary``: the reference's own Python layer is imported from PATH with its
  compiled extension ``torchmorph._C`` replaced by ``torchmorph_gb300._C`` (the
  same nine functions and signatures), so its argument handling runs unchanged
  over this package's kernels.

Nothing is written to PATH.  The exit code is pytest's.
"""

from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
import tempfile

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_API_SHIM = '''
import importlib
import sys

sys.path.insert(0, {repo!r})
import torchmorph_gb300

sys.modules["torchmorph"] = torchmorph_gb300
for name in ("morphology", "morphology.binary", "morphology.grey", "morphology.structure",
             "distance_transform", "optimal_transport", "_validation"):
    sys.modules["torchmorph." + name] = importlib.import_module("torchmorph_gb300." + name)
'''

_BOUNDARY_SHIM = '''
import sys

sys.path.insert(0, {repo!r})
from torchmorph_gb300 import _C

sys.modules["torchmorph._C"] = _C
sys.path.insert(0, {pkg!r})
import torchmorph

assert torchmorph.__file__.startswith({pkg!r}), torchmorph.__file__
'''


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--reference", required=True, help="torchmorph checkout (test/ and torchmorph/)")
    ap.add_argument("--mode", choices=("api", "boundary"), default="api")
    args, rest = ap.parse_known_args(argv)
    ref = os.path.abspath(args.reference)
    tests = os.path.join(ref, "test")
    if not os.path.isdir(tests):
        ap.error(f"{tests} is not a directory")
    with tempfile.TemporaryDirectory(prefix="tm_refsuite_") as tmp:
        suite = os.path.join(tmp, "suite")
        shutil.copytree(tests, suite, ignore=shutil.ignore_patterns("__pycache__", "*.pyc"))
        if args.mode == "api":
            shim = _API_SHIM.format(repo=REPO)
        else:
            pkg = os.path.join(tmp, "pkg")
            shutil.copytree(os.path.join(ref, "torchmorph"), os.path.join(pkg, "torchmorph"),
                            ignore=shutil.ignore_patterns("csrc", "__pycache__", "*.pyc", "*.so"))
            shim = _BOUNDARY_SHIM.format(repo=REPO, pkg=pkg)
        with open(os.path.join(suite, "conftest.py"), "w") as f:
            f.write(shim)
        with open(os.path.join(tmp, "pytest.ini"), "w") as f:
            f.write("[pytest]\nmarkers =\n    nd: N-D tests\n    bfdt: brute-force DT tests\n    cuda: CUDA tests\n")
        cmd = [sys.executable, "-m", "pytest", suite, "-c", os.path.join(tmp, "pytest.ini"),
               "--rootdir", tmp, "-p", "no:cacheprovider", "-q", *rest]
        return subprocess.call(cmd, cwd=tmp)


if __name__ == "__main__":
    sys.exit(main())
