"""Build libngg.so in-tree (sm_103a) with nvcc; translation units compile in parallel."""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libngg.so')
SOURCES = ['grid_ps.cu', 'weights.cu', 'fft.cu', 'degrid.cu', 'gcf.cu', 'gcf_grid_lo.cu', 'gcf_grid_mid.cu', 'gcf_grid_hi.cu', 'mlp.cu', 'mlp_tc.cu', 'rotate.cu', 'clean.cu', 'ngg_core.cu']
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']


def _cuda_home():
    for c in (os.environ.get('CUDA_HOME'), '/usr/local/cuda'):
        if c and os.path.exists(os.path.join(c, 'bin', 'nvcc')):
            return c
    return '/usr/local/cuda'


def _newest_input():
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, 'include', 'ngg.h'),
                                                                 os.path.abspath(__file__)]
    return max(os.path.getmtime(p) for p in paths if os.path.exists(p))


def build(force=False, verbose=False):
    """Compile every CUDA source for sm_103a and link libngg.so (returns its path)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest_input():
        return LIB
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, 'bin', 'nvcc')
    os.makedirs(BUILD, exist_ok=True)
    inc = ['-I' + os.path.join(ROOT, 'include'), '-I' + os.path.join(cuda, 'include', 'cccl')]
    flags = ARCH + ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '--expt-relaxed-constexpr'] + inc
    procs = []
    objs = []
    for src in SOURCES:
        obj = os.path.join(BUILD, src.replace('.cu', '.o'))
        objs.append(obj)
        cmd = [nvcc] + flags + ['-c', os.path.join(CSRC, src), '-o', obj]
        if verbose:
            print(' '.join(cmd))
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((src, out.decode(errors='replace')))
        elif verbose and out:
            print(out.decode(errors='replace'))
    if failed:
        msg = '\n'.join(f'--- {s}\n{o}' for s, o in failed)
        raise RuntimeError('nvcc failed:\n' + msg)
    tmp = LIB + '.tmp'
    cmd = [nvcc, '-shared'] + ARCH + objs + ['-lcufft', '-o', tmp]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose=True))
