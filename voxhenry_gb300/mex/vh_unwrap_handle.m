function ws = vh_unwrap_handle(fh, target)
% The workspace of the anonymous function that calls `target` (e.g. 'lse_matvect_mult') under the
% wrappers VoxHenry_executer.m:287-297 puts around it (@(J)fACPU(J) -> @(J)lse_matvect_mult(J, ...)),
% or [] when fh is not of that form.
ws = [];
for depth = 1:4
    if ~isa(fh, 'function_handle')
        return;
    end
    f = functions(fh);
    if ~strcmp(f.type, 'anonymous')
        return;
    end
    w = f.workspace{1};
    if ~isempty(strfind(func2str(fh), [target '(']))
        ws = w;
        return;
    end
    names = fieldnames(w);
    inner = [];
    for k = 1:numel(names)
        if isa(w.(names{k}), 'function_handle')
            inner = w.(names{k});
        end
    end
    if isempty(inner)
        return;
    end
    fh = inner;
end
end
