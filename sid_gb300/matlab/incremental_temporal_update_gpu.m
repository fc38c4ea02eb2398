function [timeseries, Varg] = incremental_temporal_update_gpu(forward_model, indir, bg_spatial, Junk_size, ...
    x_offset, y_offset, dx, Nnum, opts)
% Drop-in for incremental_temporal_update_gpu.m (same signature): frames are
% read from indir in name order, rectified (ImageRect), divided by the
% per-frame baseline and demixed chunk by chunk with the pseudo-inverse
% extraction in libsid (Q = inv(F F') F applied as inv(F F') (F Y)).  The
% reference's non-negative branch is broken (its LS_nnls call passes outputs
% LS_nnls does not return) and is not offered.
if ~exist(indir, 'dir'), disp('indir does not exist'); timeseries = []; Varg = []; return; end
files = dir(fullfile(indir, '/*.tif*'));
[~, order] = sort({files(:).name});
files = files(order);
if nargin < 9, opts = struct; end
if ~isfield(opts, 'do_crop'), opts.do_crop = 0; end
Varg = ones(1, length(files));
if isfield(opts, 'frame')
    opts.frame.end = min(opts.frame.end, length(files));
    Varg(opts.frame.start:opts.frame.step:opts.frame.end) = 0;
    line = find(Varg);
    files = files(logical(Varg));
else
    line = 1:length(files);
end
if isfield(opts, 'baseline') && ~isempty(opts.baseline)
    baseline = interp1(find(~Varg)', opts.baseline, line', 'linear', 'extrap');
else
    baseline = ones(1, length(files));
end
num = length(files);
F = single(full(forward_model));
if ~isempty(bg_spatial), F = [F; single(bg_spatial(:)')]; end
h = sid_mex('pinv_create', gpuArray(F));
cleanup = onCleanup(@() sid_mex('pinv_destroy', h));
timeseries = zeros(size(F, 1), num);
for c0 = 1:Junk_size:num
    idx = c0:min(c0 + Junk_size - 1, num);
    for k = idx
        img = ImageRect(double(imread(fullfile(indir, files(k).name), 'tiff')), x_offset, y_offset, dx, Nnum, 0);
        if opts.do_crop
            img = img(opts.crop.x_min + 1:opts.crop.x_max, opts.crop.y_min + 1:opts.crop.y_max);
        end
        if k == idx(1), Y = zeros(numel(img), numel(idx), 'single'); end
        Y(:, k - idx(1) + 1) = single(img(:));
    end
    if isfield(opts, 'idx'), Y = Y(opts.idx, :); end
    T = sid_mex('pinv_apply', h, gpuArray(Y), gpuArray(single(baseline(idx))));
    timeseries(:, idx) = double(gather(T));
end
end
