function [x, resSqAll, mseAll, xnormAll, xdiffAll, stopThresh, status] = cgne(Ain, bin, x0, NitMax, opt, gam, Rin, W)
% Drop-in for iterativeSolvers/cgne.m.  When A is opFunc = @(x,transp)
% mrSampFunc(x,transp,S,R) with S a GB300 nufftOp / sampHighOrder and R a GB300
% rcvrOp, the whole solve runs on the device (matmri_mex 'cgne'); otherwise
% the reference implementation on the path is called unchanged.
if nargin < 3, x0 = []; end
if nargin < 4 || isempty(NitMax), NitMax = 1000; end
if nargin < 5, opt = struct(); end
if nargin < 6, gam = []; end
if nargin < 7, Rin = []; end
if nargin < 8, W = []; end
S = []; R = [];
if isa(Ain, 'function_handle')
    ws = functions(Ain);
    if isfield(ws, 'workspace') && ~isempty(ws.workspace)
        vars = ws.workspace{1};
        names = fieldnames(vars);
        for k = 1:numel(names)
            v = vars.(names{k});
            if isa(v, 'nufftOp') || isa(v, 'sampHighOrder'), S = v; end
            if isa(v, 'rcvrOp'), R = v; end
        end
    end
elseif isa(Ain, 'nufftOp') || isa(Ain, 'sampHighOrder')
    S = Ain;
end
if isempty(S) || ~isprop(S, 'h') || ~isempty(gam)
    ref = fullfile(fileparts(which('mrSampFunc')), '..', 'iterativeSolvers');
    old = cd(ref); c = onCleanup(@() cd(old));
    [x, resSqAll, mseAll, xnormAll, xdiffAll, stopThresh, status] = cgne(Ain, bin, x0, NitMax, opt, gam, Rin, W);
    return;
end
if isa(S, 'nufftOp'), hn = S.h.ptr; hs = uint64(0); imDims = S.imgN; else, hn = uint64(0); hs = S.h.ptr; imDims = S.imSize; end
if isempty(R), hr = uint64(0); else, hr = R.h.ptr; end
[x, resSqAll, mseAll, xnormAll, xdiffAll, stopThresh, status] = ...
    matmri_mex('cgne', hn, hs, hr, bin, x0, NitMax, opt, W, imDims);
end
