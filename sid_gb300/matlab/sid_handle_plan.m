function [plan, kernel] = sid_handle_plan(fh, X, Y)
% SID_HANDLE_PLAN  The libsid plan behind a projector handle built the way
% reconstruct_S.m and generate_LFM_library_GPU.m build them:
%   @(V) forwardProjectGPU(H, V), @(P) backwardProjectGPU_new(H, P),
%   @(V) forwardProjectACC(psf.H, V, psf.CAindex), @(P) backwardProjectACC_new(...),
% and their neuron-kernel compositions @(V) forwardFUN_raw(convn(V, kern, 'same')).
% The captured variables of the anonymous function name the PSF (and the
% kernel).  plan = [] when fh is none of these.
plan = []; kernel = [];
info = functions(fh);
if ~isfield(info, 'workspace') || isempty(info.workspace), return; end
ws = info.workspace{1};
names = fieldnames(ws);
for k = 1:numel(names)
    if isa(ws.(names{k}), 'function_handle')
        % a composition: the raw projector inside, the kernel beside it
        plan = sid_handle_plan(ws.(names{k}), X, Y);
        for j = 1:numel(names)
            v = ws.(names{j});
            if (isnumeric(v) || isa(v, 'gpuArray')) && any(strcmp(names{j}, {'kern', 'kernel'}))
                kernel = single(gather(v));
            end
        end
        return;
    end
end
H = []; CA = [];
for k = 1:numel(names)
    v = ws.(names{k});
    if (isnumeric(v) || isa(v, 'gpuArray')) && ndims(v) >= 4, H = v; end
    if isstruct(v) && isfield(v, 'H')
        H = v.H;
        if isfield(v, 'CAindex'), CA = v.CAindex; end
    end
end
if isempty(H), return; end
if contains(func2str(fh), 'ACC'), ca = CA; else, ca = []; end
plan = sid_plan_for(H, ca, X, Y);
end
