function Backprojection = backwardProjectGPU_new(H, projection)
% Drop-in for backwardProjectGPU_new.m (same signature), in the projection
% form sid_method() selects.
plan = sid_plan_for(H, [], size(projection, 1), size(projection, 2));
Backprojection = sid_mex('adjoint', plan, single(projection), sid_method());
end
