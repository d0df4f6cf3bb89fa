"""Build the covgpu shared library in-tree with nvcc (sm_103a only).

``python -m covasim_gb300.build`` or ``covasim_gb300.build.build()``.
The library is plain C ABI over the CUDA runtime (no torch headers), so the
build is one nvcc call of a few seconds. ``-fmad=false`` keeps every float32
and float64 product separately rounded, as numpy rounds it.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, 'csrc')
INCLUDE = os.path.join(ROOT, 'include')
LIB_NAME = 'libcovgpu.so'
LIB_PATH = os.path.join(HERE, LIB_NAME)
SOURCES = ['covgpu.cu', 'covgpu_reference.cu', 'covgpu_testing.cu', 'covgpu_pop.cu', 'covgpu_dropin.cu']
OBJ_DIR = os.path.join(HERE, '_build')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']


def nvcc_path():
    cand = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not os.path.exists(cand):
        raise RuntimeError('nvcc not found: the CUDA toolkit is required to build covgpu')
    return cand


def nvcc_flags(extra=()):
    return ['-O3', '-std=c++17', '-lineinfo', '-fmad=false', '-Xcompiler', '-fPIC',
            '-I', INCLUDE, '-I', CSRC, *ARCH, *extra]


def build(verbose=False, force=False, extra=()):
    """Compile each translation unit in parallel (nvcc -c), then link the shared library."""
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    deps = srcs + [os.path.join(CSRC, f) for f in ('covgpu_device.cuh', 'covgpu_ff.cuh', 'covgpu_tables.h',
                                                   'covgpu_scan.cuh', 'covgpu_launch.cuh', 'covgpu_imm.cuh')]
    deps += [os.path.join(INCLUDE, 'covgpu.h'), __file__]
    if not force and os.path.exists(LIB_PATH):
        lib_m = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(d) <= lib_m for d in deps):
            return LIB_PATH
    os.makedirs(OBJ_DIR, exist_ok=True)
    nvcc = nvcc_path()
    objs, procs = [], []
    for src in srcs:
        obj = os.path.join(OBJ_DIR, os.path.basename(src) + '.o')
        cmd = [nvcc, *nvcc_flags(extra), '-c', '-o', obj, src]
        if verbose:
            print(' '.join(cmd))
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)))
        objs.append(obj)
    for cmd, p in procs:
        out, err = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f'nvcc failed ({p.returncode}): {" ".join(cmd)}\n{out}\n{err}')
        if verbose and (out or err):
            print(out, err)
    tmp = LIB_PATH + '.tmp'
    cmd = [nvcc, '--shared', *ARCH, '-o', tmp, *objs, '-lcudart']
    if verbose:
        print(' '.join(cmd))
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f'nvcc link failed ({res.returncode}):\n{res.stdout}\n{res.stderr}')
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == '__main__':
    extra = sys.argv[1:]
    print(build(verbose=True, force=True, extra=extra))
