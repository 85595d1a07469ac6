function [cc_sum] = fast_matched_filter_gb300(templates, moveouts, weights, data, step, varargin)
% FAST_MATCHED_FILTER_GB300  Network-summed correlation coefficients on the GPU.
%
% The MATLAB front-end of libfmf_gb300, with the arguments and layouts of the
% reference's fast_matched_filter.m:
%
%   templates  4-D [time x components x stations x templates]
%   moveouts   3-D [components x stations x templates], or 2-D
%              [stations x templates] (the same moveout for every component)
%   weights    3-D or 2-D, as moveouts
%   data       3-D [time x components x stations]
%   step       samples between two correlations
%
% Options (name, value pairs):
%   'normalize'  'short' (default) or 'full' (window mean removed)
%   'precision'  'fp32' (default; the FP32 CUDA-core form), 'split_bf16'
%                (tensor cores, bf16 hi + lo), 'auto' (split_bf16 where its
%                error bound keeps every output within 1e-5, else fp32) or
%                'bf16'
%
% Output: 2-D [lags (step apart) x templates], single.  The reference's
% 'cpu' and 'precise' archs are its CPU libraries; this front-end runs the
% GPU library through the MEX gateway fmf_gb300_mex (fmf_gb300_mex.c).

p = inputParser;
addParameter(p, 'normalize', 'short');
addParameter(p, 'precision', 'fp32');
parse(p, varargin{:});
switch p.Results.normalize
    case 'short', normalize = 0;
    case 'full', normalize = 1;
    otherwise, error('normalize must be short or full');
end
switch p.Results.precision
    case 'fp32', precision = 0;
    case 'split_bf16', precision = 1;
    case 'bf16', precision = 2;
    case 'auto', precision = 3;
    otherwise, error('precision must be fp32, split_bf16, auto or bf16');
end

n_samples_template = size(templates, 1);
n_components = size(templates, 2);
n_stations = size(templates, 3);
n_templates = size(templates, 4);
n_samples_data = size(data, 1);
n_corr = floor((n_samples_data - n_samples_template) / step + 1);

% energies of the template traces, in the templates' own precision, then single
sum_square_templates = squeeze(sum(templates .^ 2, 1));

% 2-D moveouts / weights: the same value for every component
b = ones(n_components, 1);
if numel(moveouts) ~= n_components * n_stations * n_templates
    moveouts = reshape(kron(moveouts, b), [n_components, n_stations, n_templates]);
end
if numel(weights) ~= n_components * n_stations * n_templates
    weights = reshape(kron(weights, b), [n_components, n_stations, n_templates]);
end

cc_sum = fmf_gb300_mex(single(templates(:)), single(sum_square_templates(:)), ...
                       int32(moveouts(:)), single(data(:)), single(weights(:)), ...
                       double(step), double(n_samples_template), double(n_samples_data), ...
                       double(n_templates), double(n_stations), double(n_components), ...
                       double(n_corr), double(normalize), double(precision));
cc_sum = reshape(cc_sum, [], n_templates);

% the reference wrapper's diagnostic: zeros in the first template's valid lags
n_zeros = sum(cc_sum(1:(n_corr - max(moveouts(:))), 1) == 0.);
if n_zeros > 10
    fprintf(['%d correlation computations were skipped. Can be caused by zeros in data, ' ...
             'or too low amplitudes (try to increase the gain).\n'], n_zeros);
end
end
