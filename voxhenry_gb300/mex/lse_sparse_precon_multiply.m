function JOut_full_out = lse_sparse_precon_multiply(JOut_full_in, Ae, nodeid_4_grnd, nodeid_4_injectcurr, prectol)
% Drop-in for src_lse_formation/lse_sparse_precon_multiply.m:1 on the GB300 (the factor prepared by
% lse_sparse_precon_prepare).  prectol: the inner tolerance of 'schur_gmres'.
if nargin < 5
    prectol = [];
end
JOut_full_out = voxhenry_gpu_mex('precon_multiply', JOut_full_in, prectol);
end
