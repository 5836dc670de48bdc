classdef rcvrOp
    % Drop-in for operators/@rcvrOp with precomputed maps (isCalDat = 0):
    % R = rcvrOp(maps, 0); R*x, R'*y (rcvrOp.m:104-159).
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
            if nargin < 1, error('rcvrOp:tests', 'self-tests live in the repository test suite'); end
            if isCalDat, error('rcvrOp:calibration', 'calibration from low-res data is not supported: pass precomputed maps'); end
            obj.maps = input;
            obj.imgN = size(input);
            obj.h = mmrHandle(matmri_mex('rcvr_create', input), 'rcvr');
        end
        function obj = ctranspose(obj)
            obj.adjoint = xor(obj.adjoint, 1);
        end
        function y = mtimes(obj, x)
            if obj.adjoint, outDims = obj.imgN(1:end-1); else, outDims = obj.imgN; end
            y = matmri_mex('rcvr_apply', obj.h.ptr, double(obj.adjoint), x, outDims);
        end
    end
end
