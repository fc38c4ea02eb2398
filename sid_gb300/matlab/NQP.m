function [x, w, info] = NQP(Q, b, opts)
% Drop-in for NQP.m (same signature): argmin_{x >= 0} 0.5 x'Qx + b'x by the
% Lawson-Hanson active set with the default options (no Order, Tol 0, the
% default iteration cap), solved by libsid (sid_nqp_batched, FP64).
% reg_nnls.m and the spatial update reach it through this name; other fields
% of opts (reg_nnls passes its own; this NQP.m has no Accy) are ignored, as
% NQP.m ignores them.
if nargin > 2 && isstruct(opts)
    if isfield(opts, 'Order') || (isfield(opts, 'Tol') && opts.Tol ~= 0) || isfield(opts, 'Iter')
        error('sid:nqp', 'NQP: only the default options are supported');
    end
end
[x, w, it] = sid_mex('nqp', gpuArray(double(Q)), gpuArray(double(b(:))));
x = gather(x); w = gather(w);
info.iter = double(gather(it));
end
