function [S, T] = S_update(Y, S, T, opts)
% Drop-in for S_update.m (same signature): one projected-gradient step on S
% computed by libsid (sid_s_update).  opts.lamb_spat_TV must be 0 (the
% reference's term calls an undefined 'laplace').
cls = class(S);
o = opts;
if isfield(o, 'Y'), o.Y = gpuArray(single(o.Y)); end
if isfield(o, 'hilf'), o.hilf = gpuArray(single(o.hilf)); end
[S, T] = sid_mex('s_update', gpuArray(single(Y)), gpuArray(single(S)), gpuArray(single(T)), o);
S = cast(gather(S), cls); T = cast(gather(T), cls);
end
