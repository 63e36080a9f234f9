// hos_face_impl.cuh -- host launchers of the face kernels of one WENO-AO order, included by
// hos_face5.cu, hos_face7.cu and hos_face9.cu (one translation unit per order, compiled in
// parallel).
#pragma once
#include "hos_launch.h"

namespace hos {

// PLAIN: the non-DF WENO5-AO kernels (ORDER 5; no gated form)
template <int ORDER, bool PLAIN = false>
struct FaceLaunch {
    // precision: 0 FP64, 1 FP32, 2 FP32 with the learned gate, 3 FP64 and 4 FP32 with the
    // Navier-Stokes collision time
    template <class T, int DIR, bool GATED, bool NS = false>
    static cudaError_t one(const FaceArgs& a, const Geometry& geo, cudaStream_t s, const CUtensorMap* tm) {
        using S = FaceSmem<T, ORDER, KernelTile<ORDER>>;
        const int nodeN = DIR == 0 ? geo.nodex : geo.nodey;
        const int nodeT = DIR == 0 ? geo.nodey : geo.nodex;
        if constexpr (sizeof(T) == 4) {
            if (tm) {
                using TS = TmaTile<ORDER>;
                using ST = FaceSmem<float, ORDER, TS>;
                dim3 g((nodeT + TS::T - 1) / TS::T, (nodeN + 1 + TS::N - 1) / TS::N);
                face_kernel_tma<ORDER, DIR, GATED, NS, PLAIN>
                    <<<g, FACE_THREADS, GATED ? ST::gated_bytes : ST::bytes, s>>>(a, geo, tm[DIR]);
                return cudaGetLastError();
            }
        }
        using KT = KernelTile<ORDER>;
        dim3 grid((nodeT + KT::T - 1) / KT::T, (nodeN + 1 + KT::N - 1) / KT::N);
        const size_t smem = GATED ? S::gated_bytes : S::bytes;
        face_kernel<T, ORDER, DIR, GATED, NS, PLAIN><<<grid, FACE_THREADS, smem, s>>>(a, geo);
        return cudaGetLastError();
    }

    // dynamic shared memory above 48 KB must be enabled per kernel on the current device; the
    // carveout asks for the largest shared-memory share of L1 so several tiles can be resident
    template <class K>
    static cudaError_t attrs(K k, size_t smem) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                                             (int)cudaSharedmemCarveoutMaxShared);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        return e;
    }
    template <class T, int DIR, bool GATED, bool NS = false>
    static cudaError_t configure_one() {
        using S = FaceSmem<T, ORDER, KernelTile<ORDER>>;
        const size_t smem = GATED ? S::gated_bytes : S::bytes;
        cudaError_t e = attrs(face_kernel<T, ORDER, DIR, GATED, NS, PLAIN>, smem);
        if constexpr (sizeof(T) == 4) {
            using ST = FaceSmem<float, ORDER, TmaTile<ORDER>>;
            if (e == cudaSuccess)
                e = attrs(face_kernel_tma<ORDER, DIR, GATED, NS, PLAIN>, GATED ? ST::gated_bytes : ST::bytes);
        }
        return e;
    }
    template <class T, bool GATED, bool NS = false>
    static cudaError_t configure_pair() {
        cudaError_t e = configure_one<T, 0, GATED, NS>();
        return e == cudaSuccess ? configure_one<T, 1, GATED, NS>() : e;
    }
    static cudaError_t configure(int precision) {
        switch (precision) {
            case 0: return configure_pair<double, false>();
            case 1: return configure_pair<float, false>();
            case 3: return configure_pair<double, false, true>();
            case 4: return configure_pair<float, false, true>();
            default:
                if constexpr (PLAIN) return cudaErrorInvalidValue;
                else return configure_pair<float, true>();
        }
    }

    template <class T, bool GATED, bool NS = false>
    static cudaError_t pair(const FaceArgs& ax, const FaceArgs& ay, const Geometry& geo, cudaStream_t s,
                            cudaEvent_t* ev, const CUtensorMap* tm) {
        cudaError_t e;
        if ((e = one<T, 0, GATED, NS>(ax, geo, s, tm)) != cudaSuccess) return e;
        if (ev) cudaEventRecord(ev[0], s);
        if ((e = one<T, 1, GATED, NS>(ay, geo, s, tm)) != cudaSuccess) return e;
        if (ev) cudaEventRecord(ev[1], s);
        return cudaSuccess;
    }
    static cudaError_t launch(int precision, const FaceArgs& ax, const FaceArgs& ay, const Geometry& geo,
                              cudaStream_t s, cudaEvent_t* ev, const CUtensorMap* tm) {
        switch (precision) {
            case 0: return pair<double, false>(ax, ay, geo, s, ev, nullptr);
            case 1: return pair<float, false>(ax, ay, geo, s, ev, tm);
            case 3: return pair<double, false, true>(ax, ay, geo, s, ev, nullptr);
            case 4: return pair<float, false, true>(ax, ay, geo, s, ev, tm);
            default:
                if constexpr (PLAIN) return cudaErrorInvalidValue;
                else return pair<float, true>(ax, ay, geo, s, ev, tm);
        }
    }
};

}  // namespace hos
