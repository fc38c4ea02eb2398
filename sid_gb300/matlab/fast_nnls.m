function [xx, Q, df, h] = fast_nnls(A, Y, opts, Q, df, h)
% Drop-in for fast_nnls.m (temporal_SID_update.m:45): batched NNLS on the
% normalised Gram in libsid.  Returns the solution and the normalised Gram;
% df and h are returned empty (the reference returns them only for reuse).
if nargin < 3, opts = struct; end
[xx, Q] = sid_mex('fast_nnls', gpuArray(single(A)), gpuArray(single(Y)), opts);
xx = double(gather(xx)); Q = double(gather(Q)); df = []; h = [];
end
