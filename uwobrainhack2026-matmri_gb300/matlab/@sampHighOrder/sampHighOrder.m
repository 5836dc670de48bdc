classdef sampHighOrder
    % Drop-in for operators/@sampHighOrder (approaches 0/2/3: direct sums):
    % S = sampHighOrder(b0, sampTimes, phs_spha, phs_conc, phs_grid, imMask, ...),
    % S*x, S'*y, S.setPhiDiv(ksphaDiv, kconcDiv) (sampHighOrder.m:590-622),
    % S.updateObj(...) (889-934) and the readable phase S.kbase [V x M]
    % (prepForDirect, 496-588; read by mrSampFuncMat.m:35).  Host arrays and
    % gpuArrays are both accepted.
    properties
        useSingle = 0;
        useGPU = 1;
        approach = 0;
    end
    properties (Dependent)
        kbase;
    end
    properties (SetAccess = protected)
        adjoint = 0;
        imSize = [];
        kSize = [];
        b0 = [];
        sampTimes = [];
        phs_spha = [];
        phs_conc = [];
        phs_grid = [];
        b0mask = [];
        ksphaDiv = [];
        kconcDiv = [];
        h = [];          % mmrHandle of this encoding
        baseH = [];      % with phiDiv: the handle of the base encoding, kept alive
    end
    methods
        function obj = sampHighOrder(b0, sampTimes, phs_spha, phs_conc, phs_grid, b0mask, useGPU, useSingle, approach, opt) %#ok<INUSD>
            if nargin == 0
                obj.tests();      % no inputs: self-tests (sampHighOrder.m:130-133)
                return;
            end
            if nargin < 6, b0mask = []; end
            if nargin > 6 && ~isempty(useGPU), obj.useGPU = useGPU; end
            if nargin > 7 && ~isempty(useSingle), obj.useSingle = useSingle; end
            if nargin > 8 && ~isempty(approach)
                if approach == 1
                    error('matmri:gb300:unsupported', ['approach 1 (interpolated) is not available in this class: ' ...
                        'its factors come from matmri_gb300.sho_interp.prep_for_interp and mmr_sho_interp_create']);
                end
                obj.approach = approach;
            end
            obj.b0 = gather(b0);
            obj.sampTimes = gather(sampTimes);
            obj.phs_spha = gather(phs_spha);
            obj.phs_conc = gather(phs_conc);
            obj.phs_grid = struct('x', gather(phs_grid.x), 'y', gather(phs_grid.y), 'z', gather(phs_grid.z));
            obj.b0mask = gather(b0mask);
            obj.imSize = size(obj.phs_grid.x);
            if numel(obj.imSize) == 2 && obj.imSize(2) == 1, obj.imSize = obj.imSize(1); end
            obj.kSize = size(obj.sampTimes);
            if numel(obj.kSize) == 2 && obj.kSize(2) == 1, obj.kSize = obj.kSize(1); end
            obj.h = obj.newPlan();
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
            onGPU = isa(x, 'gpuArray');
            if onGPU
                wasDouble = strcmp(classUnderlying(x), 'double');
                x = complex(single(x));
            end
            y = matmri_mex('sho_apply', obj.h.ptr, double(obj.adjoint), x, outDims, prod(extra));
            if onGPU && wasDouble, y = double(y); end
        end
        function v = get.kbase(obj)
            % [numel(b0) x numel(sampTimes)] FP64, the phase of prepForDirect (of the base encoding
            % when phiDiv is set, as the reference keeps it)
            v = matmri_mex('sho_kbase', obj.h.ptr, prod(obj.imSize), prod(obj.kSize));
        end
        function obj = setPhiDiv(obj, ksphaDiv, kconcDiv)
            % a copy whose forward is (1i*exp(1i*kbase).*phiDiv).'*x/sqrt(V) (sampHighOrder.m:374-381);
            % ksphaDiv [nspha x M], kconcDiv [nconc x M] are temporal derivatives of phs_spha, phs_conc
            if isempty(obj.baseH), base = obj.h; else, base = obj.baseH; end
            ks = double(gather(ksphaDiv));
            kc = double(gather(kconcDiv));
            if ~isempty(ks), ks = reshape(ks, size(ks, 1), []); end
            if ~isempty(kc), kc = reshape(kc, size(kc, 1), []); end
            obj.baseH = base;
            obj.h = mmrHandle(matmri_mex('sho_phidiv_create', base.ptr, ks, kc), 'sho');
            obj.ksphaDiv = ks;
            obj.kconcDiv = kc;
        end
        function obj = updateObj(obj, phs_spha, phs_conc, b0map, b0mask, phs_grid) %#ok<INUSD>
            % the reference rebuilds only the interpolated approach (sampHighOrder.m:935-954)
            error('this case not yet coded');
        end
    end
    methods (Access = private)
        function hh = newPlan(obj)
            hh = mmrHandle(matmri_mex('sho_create', obj.b0, obj.sampTimes, ...
                reshape(obj.phs_spha, size(obj.phs_spha, 1), []), reshape(obj.phs_conc, size(obj.phs_conc, 1), []), ...
                obj.phs_grid.x, obj.phs_grid.y, obj.phs_grid.z, obj.b0mask), 'sho');
        end
    end
    methods (Static, Access = private)
        function tests()
            % adjoint identity and single-precision agreement (@sampHighOrder/tests.m:10-28, 254-263)
            rng(1);
            imN = [8 8];
            kN = 64;
            grid = struct('x', randn(imN), 'y', randn(imN), 'z', randn(imN));
            S = sampHighOrder(randn(imN), randn(kN, 1) / 8, randn(16, kN), randn(4, kN), grid);
            x = complex(randn([imN 2]), randn([imN 2]));
            y = complex(randn(kN, 2), randn(kN, 2));
            lhs = sum(reshape(conj(S*x) .* y, [], 1));
            rhs = sum(reshape(conj(x) .* (S'*y), [], 1));
            assert(abs(lhs - rhs) / abs(lhs) < 1e-5, 'sampHighOrder adjoint test failed');
            E = exp(1i * S.kbase).' / sqrt(prod(imN));
            d = E * reshape(x, [], 2);
            assert(norm(reshape(S*x, [], 1) - d(:)) / norm(d(:)) < 1e-5, 'sampHighOrder direct-sum test failed');
            fprintf('sampHighOrder (GB300) self-tests passed\n');
        end
    end
end
