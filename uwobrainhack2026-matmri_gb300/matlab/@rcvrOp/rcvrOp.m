classdef rcvrOp
    % Drop-in for operators/@rcvrOp with precomputed maps (isCalDat = 0):
    % R = rcvrOp(maps, 0); R*x, R'*y (rcvrOp.m:104-159).  Host arrays and
    % gpuArrays are both accepted.
    properties
        maps = [];
        doLoop = 0;
        useGPU = 1;
    end
    properties (SetAccess = protected)
        adjoint = 0;
        imgN = [];
        h = [];
    end
    methods
        function obj = rcvrOp(input, isCalDat, apN, kalph) %#ok<INUSD>
            if nargin < 1
                obj.tests();      % no inputs: self-tests (rcvrOp.m:48-51)
                return;
            end
            if isCalDat, error('matmri:gb300:unsupported', 'calibration from low-res data is not supported: pass precomputed maps'); end
            obj.maps = input;
            obj.imgN = size(input);
            obj.h = mmrHandle(matmri_mex('rcvr_create', input), 'rcvr');
        end
        function obj = ctranspose(obj)
            obj.adjoint = xor(obj.adjoint, 1);
        end
        function y = mtimes(obj, x)
            if obj.adjoint, outDims = obj.imgN(1:end-1); else, outDims = obj.imgN; end
            onGPU = isa(x, 'gpuArray');
            if onGPU
                wasDouble = strcmp(classUnderlying(x), 'double');
                x = complex(single(x));
            end
            y = matmri_mex('rcvr_apply', obj.h.ptr, double(obj.adjoint), x, outDims);
            if onGPU && wasDouble, y = double(y); end
        end
    end
    methods (Static, Access = private)
        function tests()
            % adjoint identity (@rcvrOp/tests.m:19-31)
            rng(1);
            maps = complex(randn(16, 12, 4), randn(16, 12, 4));
            R = rcvrOp(maps, 0);
            x = complex(randn(16, 12), randn(16, 12));
            y = complex(randn(16, 12, 4), randn(16, 12, 4));
            lhs = sum(reshape(conj(R*x) .* y, [], 1));
            rhs = sum(reshape(conj(x) .* (R'*y), [], 1));
            assert(abs(lhs - rhs) / abs(lhs) < 1e-5, 'rcvrOp adjoint test failed');
            fprintf('rcvrOp (GB300) self-tests passed\n');
        end
    end
end
