function plan = sid_plan_for(H, CAindex, X, Y)
% SID_PLAN_FOR  Resident libsid projector plan for the PSF H (created on first
% use, reused while H keeps its size and contents).  CAindex = [] selects the
% uncropped PSF (forwardProjectGPU semantics).
persistent keys plans
if isempty(keys), keys = {}; plans = []; end
key = sprintf('%s|%s|%d|%d|%.17g', mat2str(size(H)), mat2str(CAindex), X, Y, double(sum(H(:))));
hit = find(strcmp(keys, key), 1);
if isempty(hit)
    if isempty(CAindex), flags = 4 + 8 + 1; else, flags = 1; end   % spectral 16-bit + 24-bit + direct / direct
    plan = sid_mex('plan', single(H), CAindex, X, Y, flags);
    keys{end+1} = key; plans(end+1) = plan;
else
    plan = plans(hit);
end
end
