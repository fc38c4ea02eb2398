function Xguess = LS_deconv(forwardFUN, backwardFUN, df, opts)
% Drop-in for LS_deconv.m (same signature): projected gradient with exact
% line search in libsid on the plan of the PSF the projector handles were
% made for (sid_handle_plan; opts.sid_plan overrides), with the lamb_TV_L2
% Laplacian term (1 x 3), lamb_L1, lamb_L2 and lamb_TV_L1's role in the step
% length.  The result comes back where df was.
if nargin < 4, opts = struct; end
if isfield(opts, 'sid_plan')
    plan = opts.sid_plan; kernel = [];
else
    [plan, kernel] = sid_handle_plan(forwardFUN, size(df, 1), size(df, 2));
end
if isempty(plan)
    error('sid:LS_deconv', ['forwardFUN/backwardFUN must be projector handles over a PSF ' ...
        '(forwardProjectGPU / forwardProjectACC and their kernel compositions), or pass opts.sid_plan']);
end
if ~isfield(opts, 'max_iter'), opts.max_iter = 8; end
if ~isfield(opts, 'lamb_L1'), opts.lamb_L1 = 0; end
if ~isfield(opts, 'lamb_L2'), opts.lamb_L2 = 0; end
if ~isfield(opts, 'lamb_TV_L1'), opts.lamb_TV_L1 = 0; end
if ~isfield(opts, 'lamb_TV_L2'), opts.lamb_TV_L2 = [0 0 0]; end
if any(opts.lamb_TV_L2) && numel(opts.lamb_TV_L2) ~= 3
    error('sid:LS_deconv', 'opts.lamb_TV_L2 needs one weight per axis (1 x 3)');
end
sid_mex('set_kernel', plan, single(kernel));
restore = onCleanup(@() sid_mex('set_kernel', plan, single([])));
ongpu = isa(df, 'gpuArray');
Xguess = sid_mex('ls_deconv_ex', plan, gpuArray(single(df)), opts.max_iter, opts.lamb_L1, opts.lamb_L2, ...
    double(opts.lamb_TV_L2), opts.lamb_TV_L1, sid_method());
if ~ongpu, Xguess = gather(Xguess); end
end
