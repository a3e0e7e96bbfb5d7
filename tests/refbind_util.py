"""Helpers of the drop-in tests: the unmodified reference package from baseline/_ref
(installed by baseline/install_reference.py) and reference systems built from plain arrays."""
import os
import sys
import tempfile

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_DIR = os.path.join(REPO, 'baseline', '_ref')


def import_reference():
    """The reference package, or None when baseline/_ref is not installed."""
    if not os.path.isdir(os.path.join(REF_DIR, 'wannierberri')):
        return None
    os.environ.setdefault('PYTHONDONTWRITEBYTECODE', '1')
    if REF_DIR not in sys.path:
        sys.path.insert(0, REF_DIR)
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter('ignore')
        import wannierberri
    return wannierberri


def ref_system(d):
    """Reference System_R (system/system_R.py) with the given lattice, R-vectors, Wannier centres
    and R-space matrices; the centres also set the MDRS shifts of its Rvectors."""
    from wannierberri.system.system_R import System_R
    from wannierberri.fourier.rvectors import Rvectors
    s = System_R(silent=True)
    s.set_real_lattice(real_lattice=d['real_lattice'])
    s.num_wann = d['XX_R']['Ham'].shape[1]
    s.set_wannier_centers(wannier_centers_cart=d['wannier_centers_cart'])
    s.rvec = Rvectors(lattice=s.real_lattice, iRvec=d['iRvec'], shifts_left_red=s.wannier_centers_red)
    for k, v in d['XX_R'].items():
        s.set_R_mat(k, np.array(v, dtype=complex))
    s.do_at_end_of_init()
    return s


def ref_run(wb, system, NKdiv, NKFFT, calculators, **kw):
    """The reference's run() without symmetry, output files in a temporary directory:
    {key: data} of the returned ResultDict."""
    from wannierberri.grid import Grid
    tmp = tempfile.mkdtemp(prefix='wbrun_')
    grid = Grid(system=system, NKdiv=NKdiv, NKFFT=NKFFT, use_symmetry=False)
    res = wb.run(system, grid=grid, calculators=calculators, parallel=False, use_irred_kpt=False, symmetrize=False,
                 fout_name=os.path.join(tmp, 'r'), file_Klist_path=os.path.join(tmp, 'k'),
                 print_progress_step_time=1e9, **kw)
    return res
