function JOut_full = lse_matvect_mult(JIn0, fN_all, Ae, z_real, z_imag, dx, idx, nodeid_4_grnd, nodeid_4_injectcurr)
% Drop-in for src_lse_formation/lse_matvect_mult.m:1 on the GB300 (libvhgpu.so through
% voxhenry_gpu_mex): the same arguments and result; the geometry (fN_all, Ae, z, idxS5) is uploaded
% once and cached by the gateway.
JOut_full = voxhenry_gpu_mex('matvec', JIn0, fN_all, Ae, z_real, z_imag, dx, idx);
end
