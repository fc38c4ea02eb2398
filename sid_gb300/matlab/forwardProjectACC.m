function TOTALprojection = forwardProjectACC(H, realspace, CAindex)
% Drop-in for forwardProjectACC.m: direct FP32 lenslet projection with the
% per-depth PSF crop CAindex.
plan = sid_plan_for(H, CAindex, size(realspace, 1), size(realspace, 2));
TOTALprojection = gather(sid_mex('forward', plan, single(realspace), 0));
end
