"""Build libmcigpu.so (the C ABI of include/mcig.h) for sm_103a with nvcc.

Translation units are compiled in parallel into mcintegratorplusplus_gb300/_build/ and linked
into mcintegratorplusplus_gb300/_build/libmcigpu.so (CUDA runtime linked statically).  Units
holding reference-order double arithmetic are compiled with -fmad=false.

    python -m mcintegratorplusplus_gb300.build [--force]
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libmcigpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# unit -> extra flags
UNITS = {
    "mcig_capi": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"],  # host sums as the device's, unfused
    "sample_generic_f64": ["-fmad=false"],
    "sample_generic_f32": [],
    "sample_generic_f32d": [],
    "sample_fast_all": [],
    "sample_fast_vec": [],
    "sample_fast_pk16": [],
    "sample_fast_pk16o": [],
    "sample_fast_pk16u": [],
    "sample_fast_pk32": [],
    "sample_fast_pk32d": [],
    "sample_fast_pk32p": [],
    "mcig_noalloc": ["-fmad=false"],
    "mcig_flow": [],
    "sample_batch": [],
    "sample_lanes": [],
    "sample_pair": [],
    "flow_accept": [],
}


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    inc = os.path.join(os.path.dirname(HERE), "include")
    files += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return max(os.path.getmtime(f) for f in files)


# flag sets tried in order when nvcc crashes.  nvcc has been seen to segfault
# intermittently on the aarch64 host when several units compile at once; a
# failed unit is retried alone, first with the same flags.
FALLBACKS = [[], [], ["-Xptxas", "-O2"], [], ["-Xptxas", "-O1"]]


def _up_to_date(unit):
    """The unit's object is newer than its source and every header it includes (the
    dependency file nvcc wrote with the object)."""
    obj = os.path.join(BUILD, unit + ".o")
    dep = os.path.join(BUILD, unit + ".d")
    if not (os.path.exists(obj) and os.path.exists(dep)):
        return False
    with open(dep) as f:
        text = f.read().replace("\\\n", " ")
    files = text.split(":", 1)[1].split() if ":" in text else []
    t = os.path.getmtime(obj)
    try:
        return all(os.path.getmtime(x) < t for x in files)
    except OSError:
        return False


def _compile(unit, flags, verbose, attempts):
    src = os.path.join(CSRC, unit + ".cu")
    obj = os.path.join(BUILD, unit + ".o")
    if _up_to_date(unit):
        return obj
    log = []
    for extra in attempts:
        cmd = [_nvcc()] + ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-v"] + \
            flags + extra + ["-MD", "-MF", os.path.join(BUILD, unit + ".d"), "-c", src, "-o", obj]
        tmp = os.path.join(BUILD, "tmp_" + unit)  # private temporary directory per unit
        os.makedirs(tmp, exist_ok=True)
        r = subprocess.run(cmd, capture_output=True, text=True, env=dict(os.environ, TMPDIR=tmp))
        log.append(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode == 0:
            break
        if verbose:
            print("nvcc failed for %s with %s (rc %d): %s" % (unit, extra, r.returncode, r.stderr[-300:]))
    with open(os.path.join(BUILD, unit + ".log"), "w") as f:
        f.write("\n".join(log))
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s" % (unit, r.stderr[-4000:]))
    if verbose:
        print("compiled", unit)
    return obj


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) > _deps():
        return LIB
    units = {u: f for u, f in UNITS.items() if os.path.exists(os.path.join(CSRC, u + ".cu"))}
    def first_try(kv):
        try:
            return _compile(kv[0], kv[1], verbose, FALLBACKS[:1])
        except RuntimeError:
            return None

    with cf.ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(first_try, units.items()))
    for i, (u, f) in enumerate(units.items()):  # retries one at a time
        if objs[i] is None:
            objs[i] = _compile(u, f, verbose, FALLBACKS[1:])
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [_nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr[-4000:])
    os.replace(tmp, LIB)
    if verbose:
        print("linked", LIB)
    return LIB


def build_plugin(src, out, verbose=False):
    """Compile a plugin source (one that ends with MCIG_PLUGIN, include/mcig/plugin.cuh) into the
    shared library `out`: the double path (-DMCIG_PLUGIN_PART=1, -fmad=false: the reference's
    operation order) and the float path (-DMCIG_PLUGIN_PART=2) as two objects, linked together.
    Skipped when `out` is newer than the source and the integrator's headers."""
    src, out = os.path.abspath(src), os.path.abspath(out)
    if os.path.exists(out) and os.path.getmtime(out) > max(os.path.getmtime(src), _deps()):
        return out
    work = out + ".build"
    os.makedirs(work, exist_ok=True)
    inc = ["-I", os.path.join(os.path.dirname(HERE), "include"), "-I", CSRC]

    def part(args):
        n, flags = args
        obj = os.path.join(work, "part%d.o" % n)
        r = None
        for extra in FALLBACKS:
            cmd = [_nvcc()] + ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC"] + inc + flags + extra + \
                ["-DMCIG_PLUGIN_PART=%d" % n, "-c", src, "-o", obj]
            r = subprocess.run(cmd, capture_output=True, text=True, env=dict(os.environ, TMPDIR=work))
            if r.returncode == 0:
                return obj
            if verbose:
                print("nvcc failed for plugin part %d with %s (rc %d)" % (n, extra, r.returncode))
        raise RuntimeError("nvcc failed for plugin %s:\n%s" % (src, r.stderr[-4000:]))

    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        objs = list(ex.map(part, [(1, ["-fmad=false"]), (2, [])]))
    tmp = out + ".tmp%d" % os.getpid()
    r = subprocess.run([_nvcc()] + ARCH + ["-shared", "-o", tmp] + objs, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("plugin link failed:\n" + r.stderr[-4000:])
    os.replace(tmp, out)
    if verbose:
        print("linked", out)
    return out


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
