function lse_sparse_precon_prepare(dx, z_real, z_imag, idxS, st_sparse_precon, nodeid_4_grnd, nodeid_4_injectcurr, Ae)
% Drop-in for src_lse_formation/lse_sparse_precon_prepare.m:1 on the GB300: the gateway keeps the
% arguments and builds the Schur-complement factor on the device when it is first applied (the
% reference keeps its factor in globals).  fl_precon_type selects the variant as in the reference
% (default 'schur_invert').
global fl_precon_type
kind = 'schur_invert';
if ~isempty(fl_precon_type)
    kind = fl_precon_type;
end
voxhenry_gpu_mex('precon_prepare', dx, z_real, z_imag, idxS, st_sparse_precon, Ae, kind);
end
