function Backprojection = backwardProjectACC_new(H, projection, CAindex)
% Drop-in for backwardProjectACC_new.m (returns double, as the reference does).
plan = sid_plan_for(H, CAindex, size(projection, 1), size(projection, 2));
Backprojection = double(gather(sid_mex('adjoint', plan, single(projection), 0)));
end
