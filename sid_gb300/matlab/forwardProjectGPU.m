function TOTALprojection = forwardProjectGPU(H, realspace)
% Drop-in for forwardProjectGPU.m (same signature): libsid projection with
% the PSF resident on the GPU, in the projection form sid_method() selects
% (default 'spectral_mixed').
plan = sid_plan_for(H, [], size(realspace, 1), size(realspace, 2));
TOTALprojection = sid_mex('forward', plan, single(realspace), sid_method());
end
