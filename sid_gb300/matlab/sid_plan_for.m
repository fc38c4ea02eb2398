function plan = sid_plan_for(H, CAindex, X, Y, batched)
% SID_PLAN_FOR  Resident libsid projector plan for the PSF H (created on first
% use and reused).  CAindex = [] selects the uncropped PSF (forwardProjectGPU
% semantics) and the storage the current sid_method() needs; a CAindex gives
% the cropped direct form (forwardProjectACC semantics).  batched = true adds
% the transposed 24-bit spectra of the tensor-core batched projections
% (SID_PLAN_SPECTRAL_TC) to the spectral forms.
% Plans are keyed on the PSF's size, the crop, the sensor size, the storage
% and a fingerprint of 4096 entries of H at fixed strided positions (a full
% pass over the 3.3 GB PSF of the 1005^2 x 31 configuration per call would
% cost more than the projection).  Two PSFs that agree at every sampled
% entry share a plan: pass distinct PSFs through sid_mex('plan', ...) directly
% when that can happen.
persistent keys plans
if isempty(keys), keys = {}; plans = []; end
flags_for = [1, 2, 4, 4 + 8, 4 + 2];   % direct, spectral_f32, _i16, _mixed, _mixed_f32
if isempty(CAindex), flags = flags_for(sid_method() + 1); else, flags = 1; end
if nargin > 4 && batched && flags ~= 1, flags = bitor(flags, 8 + 16); end
n = numel(H);
idx = unique(round(linspace(1, n, min(n, 4096))));
smp = double(gather(H(idx)));
w = (1:numel(smp))';
fp = sprintf('%.17g|%.17g|%.17g', sum(smp(:) .* w), sum(smp(:) .^ 2), smp(end));
key = sprintf('%s|%s|%d|%d|%d|%s', mat2str(size(H)), mat2str(CAindex), X, Y, flags, fp);
hit = find(strcmp(keys, key), 1);
if isempty(hit)
    plan = sid_mex('plan', single(gather(H)), CAindex, X, Y, flags);
    keys{end+1} = key; plans(end+1) = plan;
else
    plan = plans(hit);
end
end
