function [Xguess, Xguess_history] = deconvRL(forwardFUN, backwardFUN, Htf, maxIter, Xguess, opts)
% Drop-in for deconvRL.m (same signature): the ISRA iterations, in mode
% 'basic' or 'TV' (opts.lambda 1 x 3, opts.p 1 or 2), run in libsid on the
% plan of the PSF the projector handles were made for (sid_handle_plan),
% including a neuron-kernel composition; Xguess_history (maxIter x
% size(Xguess), single) when asked for.  Results come back where Xguess was.
if nargin < 6, opts = struct('lambda', 0, 'p', 1, 'mode', 'basic'); end
[plan, kernel] = sid_handle_plan(forwardFUN, size(Htf, 1), size(Htf, 2));
if isempty(plan)
    error('sid:deconvRL', ['forwardFUN/backwardFUN must be projector handles over a PSF ' ...
        '(forwardProjectGPU / forwardProjectACC and their kernel compositions)']);
end
mode = 0; if isfield(opts, 'mode') && strcmp(opts.mode, 'TV'), mode = 1; end
lam = 0; if isfield(opts, 'lambda'), lam = double(gather(opts.lambda)); end
p = 1; if isfield(opts, 'p'), p = opts.p; end
sid_mex('set_kernel', plan, kernel);
restore = onCleanup(@() sid_mex('set_kernel', plan, single([])));
ongpu = isa(Xguess, 'gpuArray');
htf = gpuArray(single(Htf)); x0 = gpuArray(single(Xguess));
if nargout > 1
    [Xguess, Xguess_history] = sid_mex('isra_ex', plan, htf, x0, maxIter, mode, p, lam, sid_method());
    Xguess_history = gather(Xguess_history);
else
    Xguess = sid_mex('isra_ex', plan, htf, x0, maxIter, mode, p, lam, sid_method());
end
if ~ongpu, Xguess = gather(Xguess); end
end
