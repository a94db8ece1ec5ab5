"""Load the reference ptychography package (Python 2 source) into this Python 3 process.

Used only by ``make_golden.py`` to produce the committed golden fixtures; nothing
else imports it and it never runs on a machine without the reference checkout.

The reference modules ``era``, ``dm``, ``forward_models`` and ``bagOfns`` are read
as text from the reference checkout, a handful of Python-2-only spellings are
rewritten, and the result is executed into fresh module objects.  The
algorithms themselves are untouched.  MPI is replaced by a single-rank fake whose
collectives are identities, which is what ``mpirun -n 1`` would do.

Rewrites (each is a pure syntax/semantics port of Python 2 behaviour):
  * ``print a, b``            -> ``print(a, b)``
  * ``np.int`` / ``np.bool``  -> ``int`` / ``bool`` (aliases removed in numpy 1.24)
  * ``np.array(a.shape)/2``   -> ``//2`` (Python 2 integer division, probe centring)
  * ``np.array(zip(...))``    -> ``np.array(list(zip(...)))`` (forward_models.py:152)
  * the ``if __name__ == '__main__'`` tail is dropped (self-tests call undefined names)

``back_projection.py`` calls ``era.psup_O_1``, which the reference never
defines; ``era.psup_O`` (the object update with that signature) is bound under
that name so the function can run.
"""
import os
import re
import sys
import types


def _reference_root():
    root = os.environ.get("PTY_REFERENCE_ROOT")
    if not root:
        raise RuntimeError("set PTY_REFERENCE_ROOT to the root of a reference checkout "
                           "(the directory holding ptychography/era.py)")
    return root


REF_ROOT = _reference_root()
PKG_DIR = os.path.join(REF_ROOT, "ptychography")


class _FakeComm:
    """Single-rank stand-in for mpi4py.MPI.COMM_WORLD."""

    def Get_rank(self):
        return 0

    def Get_size(self):
        return 1

    def bcast(self, x, root=0):
        return x

    def scatter(self, x, root=0):
        return x[0]

    def reduce(self, x, op=None, root=0):
        return x

    def allreduce(self, x, op=None):
        return x

    def Allreduce(self, src, dst, op=None):
        dst[0][...] = src[0]

    def send(self, *a, **k):
        raise RuntimeError("single rank: send unused")

    def recv(self, *a, **k):
        raise RuntimeError("single rank: recv unused")


def _install_fake_mpi():
    mpi = types.ModuleType("mpi4py.MPI")
    mpi.COMM_WORLD = _FakeComm()
    for name in ("SUM", "FLOAT", "DOUBLE", "COMPLEX", "DOUBLE_COMPLEX"):
        setattr(mpi, name, name)
    pkg = types.ModuleType("mpi4py")
    pkg.MPI = mpi
    sys.modules["mpi4py"] = pkg
    sys.modules["mpi4py.MPI"] = mpi


_PRINT_RE = re.compile(r"^(?P<pre>(?:\s*|.*?:\s*))print\s+(?!\()(?P<args>.*?)\s*(?:#.*)?$")


def _rewrite(src):
    src = src.split("if __name__ == '__main__'")[0]
    out = []
    for line in src.splitlines():
        m = _PRINT_RE.match(line)
        if m and not line.lstrip().startswith("#"):
            line = "%sprint(%s)" % (m.group("pre"), m.group("args"))
        out.append(line)
    src = "\n".join(out) + "\n"
    src = re.sub(r"np\.int\b(?!\d)", "int", src)
    src = re.sub(r"np\.bool\b(?!_)", "bool", src)
    src = src.replace("np.array(a.shape)/2", "np.array(a.shape)//2")
    src = src.replace("np.array(zip(ys.ravel(), xs.ravel()))",
                      "np.array(list(zip(ys.ravel(), xs.ravel())))")
    return src


def _load(name):
    path = os.path.join(PKG_DIR, name + ".py")
    with open(path, "r", encoding="latin-1") as f:
        src = _rewrite(f.read())
    mod = types.ModuleType(name)
    mod.__file__ = path
    sys.modules[name] = mod
    exec(compile(src, path, "exec"), mod.__dict__)
    return mod


def load_reference():
    """Return a namespace with the reference's era, dm, forward_models, bagOfns."""
    import warnings
    warnings.filterwarnings("ignore", category=SyntaxWarning)
    warnings.filterwarnings("ignore", category=DeprecationWarning)
    _install_fake_mpi()
    ns = types.SimpleNamespace()
    ns.bagOfns = _load("bagOfns")
    ns.era = _load("era")
    ns.dm = _load("dm")
    ns.forward_models = _load("forward_models")
    ns.era.psup_O_1 = ns.era.psup_O
    ns.back_projection = _load("back_projection")
    return ns
