"""Install the unmodified reference package (wannier-berri) into baseline/_ref for the drop-in tests.

    python baseline/install_reference.py [REFERENCE_ROOT]      # default: /root/reference

What it does, offline:
  1. pip install --no-index --no-build-isolation --no-deps --target baseline/_ref <a copy of the root>
     (the copy under a temporary directory keeps the build from writing into the source tree);
  2. the one pure-Python dependency the package imports at start-up and that the GPU machines lack,
     ``packaging``, from the local wheelhouse (--find-links /opt/wheelhouse, --no-deps);
  3. two stand-ins for modules the package imports but never uses on the path these tests drive:
     ``termcolor`` (cprint / colored print plain text) and ``numba`` (njit returns the function
     unchanged; the tetrahedron weights then run as plain Python).
numpy and scipy come from the interpreter.  baseline/_ref is git-ignored; it is pure Python, so the
same directory serves the x86 and the Arm machines.
"""
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
TARGET = os.path.join(HERE, '_ref')


def main(root):
    if os.path.isdir(TARGET):
        shutil.rmtree(TARGET)
    os.makedirs(TARGET)
    tmp = tempfile.mkdtemp(prefix='wbref_src_')
    src = os.path.join(tmp, 'wannier-berri')
    shutil.copytree(root, src, ignore=shutil.ignore_patterns('__pycache__', '*.pyc', 'tests', 'docs', 'examples'))
    pip = [sys.executable, '-m', 'pip', 'install', '--no-index', '--no-deps', '--target', TARGET]
    subprocess.run(pip + ['--no-build-isolation', src], check=True)
    subprocess.run(pip + ['--find-links', '/opt/wheelhouse', 'packaging'], check=True)
    shutil.rmtree(tmp, ignore_errors=True)
    os.makedirs(os.path.join(TARGET, 'termcolor'), exist_ok=True)
    with open(os.path.join(TARGET, 'termcolor', '__init__.py'), 'w') as f:
        f.write("def cprint(*a, **k):\n    print(a[0] if a else '')\n\n\n"
                "def colored(s, *a, **k):\n    return s\n")
    os.makedirs(os.path.join(TARGET, 'numba'), exist_ok=True)
    with open(os.path.join(TARGET, 'numba', '__init__.py'), 'w') as f:
        f.write("def njit(*a, **k):\n    if len(a) == 1 and callable(a[0]) and not k:\n        return a[0]\n"
                "    return lambda f: f\n\n\njit = njit\n")
    print(f"reference installed into {TARGET}")


if __name__ == '__main__':
    main(sys.argv[1] if len(sys.argv) > 1 else '/root/reference')
