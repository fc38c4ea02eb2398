function [xx, Q, df, h] = fast_nnls(A, Y, opts, Q, df, h)
% Drop-in for fast_nnls.m (same signature, every input and output):
% batched NNLS on the normalised Gram in libsid.  opts.warm_start (a matrix,
% or 1 for the inverse-Gram start), opts.total, and the caller's Q, df, h
% (fast_nnls.m:58-62) are honoured; the two-argument call uses tol = 1e-12 as
% the reference does.  df comes back with no columns except in total mode
% (the reference removes every retired column from it).
args = {};
if nargin >= 3, args{1} = opts; end
if nargin < 4 || isempty(Q), Q = []; end
if nargin < 5, df = []; end
if nargin < 6, h = []; end
if nargin >= 3 && isfield(opts, 'warm_start') && numel(opts.warm_start) > 1
    opts.warm_start = gpuArray(single(opts.warm_start)); args{1} = opts;
end
g = @(v) gpuArray(single(v));
if isempty(A), Ag = []; Yg = []; else, Ag = g(A); Yg = g(Y); end
if isempty(Q), Qg = []; hg = []; else, Qg = g(Q); hg = g(h); end
if isempty(df), dfg = []; else, dfg = g(df); end
if nargin >= 3
    [xx, Q, df, h] = sid_mex('fast_nnls_ex', Ag, Yg, args{1}, Qg, dfg, hg);
else
    [xx, Q, df, h] = sid_mex('fast_nnls_ex', Ag, Yg);
end
xx = double(gather(xx)); Q = double(gather(Q)); df = double(gather(df)); h = double(gather(h));
end
