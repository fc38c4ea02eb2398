function recon_nnmf = reconstruct_S(S, psf_ballistic, opts)
% Drop-in for reconstruct_S.m (same signature): the component images of S are
% reconstructed in libsid on the PSF's resident plan -- background clip at
% quantile opts.q of the non-microlens pixels, normalisation, back projection
% and the solve ('fast_nnls' = LS_deconv or 'ISRA' = deconvRL), with the
% neuron kernel of opts.ker_shape / opts.ker_param composed into the
% projector.  All components go to one call (sid_mex 'reconstruct_batch'),
% which runs them in groups through the batched projections -- on the tensor
% cores for the default spectral form, whose plan then carries the
% transposed spectra -- in place of the reference's parfor over components.
% TV weights route the solve through the LS_deconv shim, one component at a
% time.  Without opts.gpu_ids the reference reconstructs on the CPU with the
% cropped PSF (psf_ballistic.CAindex); the same choice selects the plan here.
if nargin < 3, opts = struct; end
dflt = struct('microlenses', zeros(size(S, 2), size(S, 3)), 'lamb_TV_L1', 0, 'lamb_TV_L2', [0 0 0], ...
    'lamb_L1', 0, 'lamb_L2', 0, 'max_iter', 8, 'gpu_ids', [], 'whichSolver', 'fast_nnls', ...
    'ker_shape', 'ball', 'maxIter', 8, 'q', 0.8);
f = fieldnames(dflt);
for k = 1:numel(f)
    if ~isfield(opts, f{k}), opts.(f{k}) = dflt.(f{k}); end
end
if isempty(opts.gpu_ids) && isfield(psf_ballistic, 'CAindex'), ca = psf_ballistic.CAindex; else, ca = []; end
tv = any(opts.lamb_TV_L2) || opts.lamb_TV_L1;
method = sid_method(); if ~isempty(ca), method = 0; end
% the tensor-core batched projections need the transposed 24-bit spectra (SID_PLAN_SPECTRAL_TC)
plan = sid_plan_for(psf_ballistic.H, ca, size(S, 2), size(S, 3), ~tv && method == 3 && size(S, 1) > 1);
if isfield(opts, 'ker_param'), kernel = single(generate_kernel(opts.ker_shape, opts.ker_param)); else, kernel = []; end
sid_mex('set_kernel', plan, kernel);
restore = onCleanup(@() sid_mex('set_kernel', plan, single([])));
recon_nnmf = cell(size(S, 1), 1);
if ~tv
    % the solve's max_iter: opts.maxIter for ISRA, opts.max_iter for LS_deconv (reconstruct_S.m:142-145)
    o = opts;
    if strcmp(opts.whichSolver, 'ISRA'), o.max_iter = opts.maxIter; end
    imgs = gpuArray(single(permute(S, [2 3 1])));
    X = sid_mex('reconstruct_batch', plan, imgs, double(opts.microlenses), o, method);
    for ii = 1:size(S, 1)
        recon_nnmf{ii} = gather(X(:, :, :, ii));
    end
    return
end
for ii = 1:size(S, 1)
    img = gpuArray(single(squeeze(S(ii, :, :))));
    % clip, normalise and back-project here, then the TV solve of the LS_deconv shim
    img = max(img - quantile(img(opts.microlenses(:) == 0), opts.q), 0);
    img = img / max(img(:));
    nrm = sqrt(sum(img(:) .^ 2));
    Htf = sid_mex('adjoint', plan, img / nrm, method);
    o = opts;
    o.lamb_L1 = min(quantile(Htf(:), 1 - 1e-4), opts.lamb_L1);
    o.sid_plan = plan;
    recon_nnmf{ii} = gather(nrm * LS_deconv([], [], Htf, o));
end
end
