function [x, flag, relres, iter, resvec] = pgmres(A, b, restart, tol, maxit, L1, L2, R1, R2, x0)
% Drop-in for src_iterative_solver/pgmres.m:70 on the GB300 for the executer's call
% (VoxHenry_executer.m:294-295): A wraps lse_matvect_mult and L1 wraps lse_sparse_precon_multiply.
% The whole restarted GMRES (left preconditioner, CGS Arnoldi, pgmres.m's stopping rule and outputs)
% runs on the device in one gateway call.  R1 alone gives right preconditioning.  Other operator
% forms (matrices, other functions, L2 / R2) are not provided.
if nargin < 6, L1 = []; end
if nargin < 7, L2 = []; end
if nargin < 8, R1 = []; end
if nargin < 9, R2 = []; end
if nargin < 10, x0 = []; end
ws = vh_unwrap_handle(A, 'lse_matvect_mult');
if isempty(ws) || ~isempty(L2) || ~isempty(R2) || (~isempty(L1) && ~isempty(R1))
    error('VoxHenryGPU:VH_ERR_UNSUPPORTED', 'pgmres on the GPU takes A = @(J)lse_matvect_mult(J, ...) and one preconditioner');
end
pc = L1;
flexible = 0;
if isempty(pc) && ~isempty(R1)
    pc = R1;
    flexible = 1;   % right preconditioning: the flexible solver with a fixed preconditioner
end
use_pc = ~isempty(pc);
if use_pc && isempty(vh_unwrap_handle(pc, 'lse_sparse_precon_multiply'))
    error('VoxHenryGPU:VH_ERR_UNSUPPORTED', 'the preconditioner must wrap lse_sparse_precon_multiply');
end
[x, flag, relres, iter, resvec] = voxhenry_gpu_mex('gmres', b, restart, tol, maxit, flexible, x0, ws.fN_all, ...
    ws.Ae, ws.z_real, ws.z_imag, ws.dx, ws.idxS5, double(use_pc));
end
