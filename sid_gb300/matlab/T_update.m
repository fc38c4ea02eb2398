function [S, T] = T_update(Y, T, S, opts)
% Drop-in for T_update.m (same signature): one projected-gradient step on T
% computed by libsid (sid_t_update).  Y may be single or half; the results
% come back in the class of the inputs.
cls = class(T);
o = opts;
if isfield(o, 'active') && ~islogical(o.active)
    m = false(size(Y, 1), 1); m(o.active) = true; o.active = m;
end
if isfield(o, 'Y'), o.Y = gpuArray(single(o.Y)); end
[S, T] = sid_mex('t_update', gpuArray(single(Y)), gpuArray(single(T)), gpuArray(single(S)), o);
S = cast(gather(S), cls); T = cast(gather(T), cls);
end
