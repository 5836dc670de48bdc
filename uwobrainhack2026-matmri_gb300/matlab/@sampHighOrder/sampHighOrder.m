classdef sampHighOrder
    % Drop-in for operators/@sampHighOrder (approaches 0/2/3: direct sums):
    % S = sampHighOrder(b0, sampTimes, phs_spha, phs_conc, phs_grid, imMask, ...).
    properties
        useSingle = 0;
        useGPU = 1;
        approach = 0;
    end
    properties (SetAccess = protected)
        adjoint = 0;
        imSize = [];
        kSize = [];
        h = [];
    end
    methods
        function obj = sampHighOrder(b0, sampTimes, phs_spha, phs_conc, phs_grid, b0mask, useGPU, useSingle, approach, opt) %#ok<INUSD>
            if nargin == 0, error('sampHighOrder:tests', 'self-tests live in the repository test suite'); end
            if nargin < 6, b0mask = []; end
            if nargin > 8 && ~isempty(approach) && approach == 1
                error('sampHighOrder:approach', ['approach 1 (interpolated) is not available in this class: ' ...
                    'its factors come from matmri_gb300.sho_interp.prep_for_interp and mmr_sho_interp_create']);
            end
            obj.imSize = size(phs_grid.x);
            if numel(obj.imSize) == 2 && obj.imSize(2) == 1, obj.imSize = obj.imSize(1); end
            obj.kSize = size(sampTimes);
            if numel(obj.kSize) == 2 && obj.kSize(2) == 1, obj.kSize = obj.kSize(1); end
            obj.h = mmrHandle(matmri_mex('sho_create', b0, sampTimes, reshape(phs_spha, size(phs_spha,1), []), ...
                reshape(phs_conc, size(phs_conc,1), []), phs_grid.x, phs_grid.y, phs_grid.z, b0mask), 'sho');
        end
        function obj = ctranspose(obj)
            obj.adjoint = xor(obj.adjoint, 1);
        end
        function y = mtimes(obj, x)
            if obj.adjoint
                extra = size(x); extra = extra(numel(obj.kSize)+1:end); outDims = [obj.imSize, extra];
            else
                extra = size(x); extra = extra(numel(obj.imSize)+1:end); outDims = [obj.kSize, extra];
            end
            if isempty(extra), extra = 1; end
            y = matmri_mex('sho_apply', obj.h.ptr, double(obj.adjoint), x, outDims, prod(extra));
        end
    end
end
