"""Recipe that builds the reference's own CPU code for the fusion path into
oracle/_ref/ (git-ignored).  Test and baseline infrastructure only.

Two steps:

1. ``stage()`` (needs the read-only reference checkout, i.e. only in the
   development container): copy the kifi sources of the path into
   ``oracle/_ref/src/kifi`` and apply the two mechanical edits that MSVC 2013
   tolerated and g++ rejects:
     * KinectFission/kifi/util/numeric.h:85,97 -- add the ``typename`` keyword
       in front of the dependent ``std::iterator_traits<...>::value_type``;
     * KinectFission/kifi/util/iterator.h:43-93 -- ``transform_iterator`` uses
       ``value_type`` / ``difference_type`` of its dependent base class
       unqualified; re-declare the five iterator typedefs at the top of the
       class body.
   No other file is changed.  The staged copy travels with the working tree,
   so the same build also works where the reference checkout is absent.

2. ``build()``: compile the staged ``.cpp`` files plus ``oracle/ref_driver.cpp``
   (a C-ABI driver around the reference classes) into
   ``oracle/_ref/libkifi_ref.so`` with g++ -O2, no fast-math, no FP
   contraction, using oracle/shim/xmmintrin.h in place of the SSE header (so
   the identical code runs on x86-64 and aarch64) and the force-included
   oracle/shim/kifi_ref_prelude.h.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def reference_root():
    """The read-only reference checkout: $KIFI_REFERENCE_ROOT when set, else a
    directory named ``reference`` beside this repository's root."""
    env = os.environ.get("KIFI_REFERENCE_ROOT")
    if env:
        return env
    return os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


REF_ROOT = reference_root()
REF_KIFI = os.path.join(REF_ROOT, "KinectFission", "kifi")
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")
LIB = os.path.join(OUT, "libkifi_ref.so")

# Translation units of the path (Integrator, Volume, Mesher, ICP, Renderer,
# DepthSensorParams, DepthStream) and the utilities they link against.
TUS = [
    "Integrator.cpp", "Volume.cpp", "Mesher.cpp", "ICP.cpp", "Renderer.cpp",
    "DepthSensorParams.cpp", "DepthStream.cpp", "Pipeline.cpp",
    "util/stop_watch.cpp", "util/fstream.cpp",
]

_ITER_TYPEDEFS = (
    "\ttypedef typename std::iterator_traits< Iterator >::value_type value_type;\n"
    "\ttypedef typename std::iterator_traits< Iterator >::difference_type difference_type;\n"
    "\ttypedef typename std::iterator_traits< Iterator >::iterator_category iterator_category;\n"
    "\ttypedef typename std::iterator_traits< Iterator >::pointer pointer;\n"
    "\ttypedef typename std::iterator_traits< Iterator >::reference reference;\n"
)


def reference_present():
    return os.path.isdir(REF_KIFI)


def stage():
    """Copy + patch the reference sources into oracle/_ref/src (idempotent)."""
    if not reference_present():
        return False
    dst = os.path.join(SRC, "kifi")
    if os.path.isdir(dst):
        shutil.rmtree(dst)
    os.makedirs(os.path.join(dst, "util"))
    for sub in ("", "util"):
        d = os.path.join(REF_KIFI, sub)
        for name in os.listdir(d):
            if name.endswith((".h", ".cpp")) and not name.startswith("windows_"):
                shutil.copyfile(os.path.join(d, name), os.path.join(dst, sub, name))
    num = os.path.join(dst, "util", "numeric.h")
    text = open(num, encoding="latin-1").read()
    text = text.replace("typedef std::iterator_traits", "typedef typename std::iterator_traits")
    open(num, "w", encoding="latin-1").write(text)
    it = os.path.join(dst, "util", "iterator.h")
    text = open(it, encoding="latin-1").read()
    cls = text.index("class transform_iterator : public std::iterator")
    pub = text.index("public:\n", cls) + len("public:\n")
    text = text[:pub] + _ITER_TYPEDEFS + text[pub:]
    open(it, "w", encoding="latin-1").write(text)
    return True


def build(verbose=False):
    """Compile oracle/_ref/libkifi_ref.so from the staged sources.

    Returns the library path, or None when no staged sources exist."""
    if reference_present():
        stage()
    if not os.path.isdir(os.path.join(SRC, "kifi")):
        return None
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    flags = [
        "-std=c++14", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
        "-w", "-DNDEBUG",
        "-I", os.path.join(HERE, "shim"), "-I", SRC,
        "-include", os.path.join(HERE, "shim", "kifi_ref_prelude.h"),
    ]
    srcs = [os.path.join(SRC, "kifi", t) for t in TUS] + [os.path.join(HERE, "ref_driver.cpp")]
    procs, objs = [], []
    for s in srcs:
        o = os.path.join(objdir, os.path.basename(s).replace(".cpp", ".o"))
        objs.append(o)
        cmd = ["g++"] + flags + ["-c", s, "-o", o]
        if verbose:
            print(" ".join(cmd))
        procs.append((subprocess.Popen(cmd), s))
    for p, s in procs:
        if p.wait() != 0:
            raise RuntimeError("reference build failed on " + s)
    subprocess.check_call(["g++", "-shared", "-o", LIB] + objs)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
