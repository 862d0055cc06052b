function [x, flag, relres, iter, resvec] = fpgmres(A, b, restart, tol, maxit, R1, R2, x0)
% Drop-in for src_iterative_solver/fpgmres.m:58 on the GB300 (flexible GMRES with the right
% preconditioner R1 wrapping lse_sparse_precon_multiply, VoxHenry_executer.m:296-297).
if nargin < 6, R1 = []; end
if nargin < 7, R2 = []; end
if nargin < 8, x0 = []; end
ws = vh_unwrap_handle(A, 'lse_matvect_mult');
if isempty(ws) || ~isempty(R2)
    error('VoxHenryGPU:VH_ERR_UNSUPPORTED', 'fpgmres on the GPU takes A = @(J)lse_matvect_mult(J, ...) and one preconditioner');
end
use_pc = ~isempty(R1);
[x, flag, relres, iter, resvec] = voxhenry_gpu_mex('gmres', b, restart, tol, maxit, 1, x0, ws.fN_all, ...
    ws.Ae, ws.z_real, ws.z_imag, ws.dx, ws.idxS5, double(use_pc));
end
