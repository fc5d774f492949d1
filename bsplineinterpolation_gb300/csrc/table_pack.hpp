// Packing of a table's per-axis device data (knots, keys, reciprocals, FP32
// knot splits, LU factors, collocation stencils) into one host staging
// buffer, and binding of the device descriptors once that buffer sits on the
// device. Used by single tables (capi.cu) and by table batches (batch.cu),
// which pack many tables into one arena.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "device_common.cuh"
#include "dw.cuh"
#include "spline_model.hpp"

namespace intp_gb300 {

// Bump allocator over one host staging buffer mirrored to one device buffer.
struct Arena {
    std::vector<unsigned char> host;
    size_t add(size_t bytes) {
        const size_t off = (host.size() + 255) & ~size_t(255);
        host.resize(off + (bytes > 0 ? bytes : 1));
        return off;
    }
    template <class T>
    size_t put(const std::vector<T>& v) {
        const size_t off = add(v.size() * sizeof(T));
        if (!v.empty()) std::memcpy(host.data() + off, v.data(), v.size() * sizeof(T));
        return off;
    }
};

// Device pointers of one axis's LU factor: FP64 (the FP64 form), FP32 (the
// mixed form's plain FP32 solve) and double-word (its default solve) copies.
struct AxisFactorDev {
    const double *lower, *upper, *dinv, *bottom, *right;
    const float *lowerf, *upperf, *dinvf, *bottomf, *rightf;
    const DW *lowerw, *upperw, *dinvw, *bottomw, *rightw;
    int64_t clo, chi;      // FP64 rows identical to row clo (LineFactor::const_lo/const_hi)
    int64_t clo32, chi32;  // the same for the FP32 rows (LineFactor::const_lo32/const_hi32)
    int64_t zside, zside32;  // cyclic side-band sums: zero entries from here (LineFactor::zside/zside32)
};

// Arena offsets of one table's per-axis arrays.
struct PackedTable {
    struct Axis {
        size_t knots, keys, rinv, rinvf, kdf, khi, klo;
        size_t lower, upper, dinv, bottom, right, lowerf, upperf, dinvf, bottomf, rightf;
        size_t lowerw, upperw, dinvw, bottomw, rightw;
    } ax[kMaxDim];
};

// Appends the per-axis arrays of `m` to the arena.
void pack_table(const TableModel& m, Arena& ar, PackedTable& pt);

// Fills the device descriptor (everything but the control-point pointer) and
// the factor pointers of a table packed at `base` on the device. lo_user[d]
// is the axis's x_min as given by the caller (the hint origin of a uniform
// axis).
void bind_table(const TableModel& m, const double* lo_user, const PackedTable& pt, const unsigned char* base,
                TableDev& dv, AxisFactorDev* fac);

// Output plan of a derivative request: nderiv rows of derivative orders,
// row k at derivs[k * row_stride], of which the first `dim` are used (NULL:
// the value only). Orders above the spline order give 0. Returns false with
// the reason in err for invalid requests.
bool build_deriv_plan(int dim, int order, const int32_t* derivs, int32_t nderiv, int row_stride, DerivPlan& plan,
                      std::string& err);

// Sets the message intp_last_error() returns on the calling thread.
void set_last_error(const std::string& msg);


}  // namespace intp_gb300
