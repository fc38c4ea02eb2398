function [X, G] = LS_nnls(A, Y, opts, G, x)
% Drop-in for LS_nnls.m for the GPU case (opts.gpu_id set): batched
% projected-gradient NNLS on libsid's tensor-core contractions.  G / x inputs
% are not forwarded by this shim (the C entry point accepts them).
if nargin < 3, opts = struct; end
[X, G] = sid_mex('ls_nnls', gpuArray(single(A)), gpuArray(single(Y)), opts);
X = double(gather(X)); G = double(gather(G));
end
