"""CPU oracle for the VoxHenry VIE solve path -- TEST INFRASTRUCTURE ONLY.

This package is a NumPy/SciPy restatement of the reference MATLAB/Octave code
(acyucel/VoxHenry) for the path that the GPU library accelerates: the input
reader, panel numbering, the incidence matrix Ae, port nodes and right-hand
sides, the circulant Green tensor, the FFT matvec, the Schur-complement
preconditioner, (F)GMRES and the Y -> Z -> R, L post-processing.

It exists to check the GPU library.  Only ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` may import it, and there only as the
checker (or as the timed CPU baseline).  The product path
(``voxhenry_gb300``) never imports it.

Pinning: the restatement is checked against the reference's own published
outputs (results_numex1_straight_conductor/data_R_jL_mat.mat: R + jL at 41
frequencies; data_curr_plot.mat: the solution vector at 2.5 GHz and the
Ae_only_leaving / Ae_only_entering_bndry matrices that fix the panel
numbering), against the FastHenry table shipped with the reference and
against the analytic DC resistance of a prism.  Compact fixtures extracted
from those files live in ``tests/golden/`` together with the script that
made them.

Third-party arithmetic: the reference factors the Schur complement with
CHOLMOD 3.0.12 (``ldlchol``/``ldlsolve``, MATLAB) or sparse LU (Octave); the
CHOLMOD sources are not part of the reference.  The oracle uses SciPy's
SuperLU (``splu``), i.e. the Octave ``lu`` semantics: any exact factorisation
gives the same preconditioner up to rounding.
"""
