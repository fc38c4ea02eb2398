function Xguess = LS_deconv(forwardFUN, backwardFUN, df, opts)
% Drop-in for LS_deconv.m when forwardFUN/backwardFUN are the libsid
% projector shims: the whole solve runs in libsid (sid_deconv_ls) on the plan
% of the PSF the handles were made for, passed as opts.sid_plan.  TV terms are
% not supported.
if nargin < 4, opts = struct; end
if ~isfield(opts, 'sid_plan')
    error('sid:LS_deconv', 'opts.sid_plan (a plan from sid_plan_for) is required');
end
if ~isfield(opts, 'max_iter'), opts.max_iter = 8; end
if ~isfield(opts, 'lamb_L1'), opts.lamb_L1 = 0; end
if ~isfield(opts, 'lamb_L2'), opts.lamb_L2 = 0; end
Xguess = sid_mex('ls_deconv', opts.sid_plan, single(df), opts.max_iter, opts.lamb_L1, opts.lamb_L2, 3);
end
