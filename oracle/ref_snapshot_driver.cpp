// ORACLE - test infrastructure only. C entry points over the reference's
// snapshot code (src/sim/snapshot.cpp, compiled unmodified from the reference
// tree by ref_build.py): key hash and name, flag hash, and the FCS1 reader and
// writer (a file is loaded and written back by the reference). The solver
// methods snapshot.cpp references are stubbed here: capture and restore are
// never called through this library.
#include <cstdio>
#include <cstring>
#include <string>

#include "lbm_solver.h"
#include "snapshot.h"

namespace foilcfd {
float* LBMSolver::activeDeviceF() { return nullptr; }
void LBMSolver::notifySnapshotRestored(bool) {}
std::size_t LBMSolver::fBufferBytes() const { return 0; }
DeviceVelocityField LBMSolver::velocityField() const { return DeviceVelocityField{}; }
GridDims LBMSolver::dims() const { return GridDims{}; }
const LatticeScaling& LBMSolver::scaling() const {
    static LatticeScaling s;
    return s;
}
const float* LBMSolver::deviceRho() const { return nullptr; }
const std::vector<std::uint8_t>& LBMSolver::hostFlags() const {
    static std::vector<std::uint8_t> v;
    return v;
}
bool LBMSolver::restoreFromMacroscopic(const float*, const float*, const float*, const float*, std::string*) {
    return false;
}
} // namespace foilcfd

namespace {
foilcfd::SnapshotKey key_of(const char* id, int bucket, float u, int nx, int ny, int nz, int ver) {
    foilcfd::SnapshotKey k;
    k.geometryId = id;
    k.aoaBucket = bucket;
    k.u_lat = u;
    k.dims.nx = nx; k.dims.ny = ny; k.dims.nz = nz;
    k.solverVersion = ver;
    return k;
}
} // namespace

extern "C" unsigned long long ref_key_hash(const char* id, int bucket, float u, int nx, int ny, int nz, int ver) {
    return key_of(id, bucket, u, nx, ny, nz, ver).hash();
}

extern "C" int ref_key_string(const char* id, int bucket, float u, int nx, int ny, int nz, int ver, char* out,
                              int cap) {
    const std::string s = key_of(id, bucket, u, nx, ny, nz, ver).toString();
    std::snprintf(out, static_cast<size_t>(cap), "%s", s.c_str());
    return static_cast<int>(s.size());
}

extern "C" int ref_bucket(float aoa) { return foilcfd::SnapshotKey::bucketForAoA(aoa); }

extern "C" unsigned long long ref_hash_flags(const unsigned char* p, unsigned long long n) {
    return foilcfd::hashFlags(p, static_cast<std::size_t>(n));
}

// Load `in` with the reference reader; on success write it back to `out`
// with the reference writer. 0, or -1 with the reader's reason in err.
extern "C" int ref_fcs_roundtrip(const char* in, const char* out, char* err, int cap) {
    foilcfd::CompactSnapshot s;
    std::string e;
    if (!s.loadFromFile(in, &e)) {
        std::snprintf(err, static_cast<size_t>(cap), "%s", e.c_str());
        return -1;
    }
    if (out && !s.saveToFile(out, &e)) {
        std::snprintf(err, static_cast<size_t>(cap), "%s", e.c_str());
        return -1;
    }
    return 0;
}
