function forward_model = generate_LFM_library_CPU(centers, psf_ballistic, r, dim, m, kernel, method)
% Drop-in for generate_LFM_library_CPU.m (same signature, plus an optional
% method): every neuron is the kernel (or, without one, the ball of radius r
% and axial radius r/dim(3)) painted at its centre, forward-projected on the
% PSF's resident plan and L2-normalised, all in one libsid call.  Returns the
% same sparse N x prod(m(1:2)) double matrix.  method 'direct' (default: FP32
% lenslet taps) or 'spectral' (tensor-core windows: faster, about 1e-5
% relative per row).
if nargin < 6, kernel = []; end
if nargin < 7 || isempty(method), method = 'direct'; end
plan = sid_plan_for(psf_ballistic.H, [], m(1), m(2));
F = sid_mex('library_kernel', plan, double(centers), double(r), double(dim), single(kernel), method);
forward_model = sparse(double(gather(F)));
end
