// Plain (host + device) types of the learned u_tau seed: parameter layout,
// normalisation constants and the device view of a network.
#pragma once

#include <cstdint>

namespace fcfd {
namespace wallnet {

constexpr int kH = 32;
constexpr int kParams = 1217;  // W1[32][3], b1[32], W2[32][32], b2[32], W3[32], b3
constexpr int kOffW1 = 0, kOffB1 = 96, kOffW2 = 128, kOffB2 = 1152, kOffW3 = 1184, kOffB3 = 1216;

/// Normalisation constants (FP32): inputs (log u_par, log y, log nu), target
/// log u_tau - log u_par.
struct Norm {
    float inMean[3], inInvStd[3];
    float outMean, outStd;
};

/// Device view of a network: BF16 parameter bits + normalisation.
struct NetDev {
    const std::uint16_t* w = nullptr;
    Norm norm{};
};

} // namespace wallnet
} // namespace fcfd
