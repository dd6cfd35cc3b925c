// Core types of the GB300 Neon API: 3-D vectors, enums and exceptions with
// the names and meaning of libNeonCore (include/Neon/core/types/*,
// Exceptions.h:19-26). Header-only; compiled by nvcc in the user's unit.
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <functional>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#if defined(__CUDACC__)
#define NEON_CUDA_HOST_DEVICE __host__ __device__
#define NEON_CUDA_DEVICE_ONLY __device__
#else
#define NEON_CUDA_HOST_DEVICE
#define NEON_CUDA_DEVICE_ONLY
#endif
#define NEON_OUT
#define NEON_IO

namespace Neon {

// ------------------------------------------------------------------ exceptions
class NeonException : public std::exception {
   public:
    explicit NeonException(std::string component = "") : mComponent(std::move(component)) {}
    template <typename T>
    NeonException& operator<<(const T& v)
    {
        std::ostringstream s;
        s << v;
        mMsg += s.str();
        return *this;
    }
    const char* what() const noexcept override
    {
        mFull = "[" + mComponent + "] " + mMsg;
        return mFull.c_str();
    }

   private:
    std::string         mComponent, mMsg;
    mutable std::string mFull;
};

#define NEON_THROW(e) throw(e)
#define NEON_THROW_UNSUPPORTED_OPERATION(msg)                                   \
    do {                                                                        \
        ::Neon::NeonException e_("UnsupportedOperation");                       \
        e_ << msg << " (" << __FILE__ << ":" << __LINE__ << ")";                \
        throw e_;                                                               \
    } while (0)
#define NEON_DEV_UNDER_CONSTRUCTION(msg) NEON_THROW_UNSUPPORTED_OPERATION("under construction: " << msg)

// ------------------------------------------------------------------ vectors
template <typename T>
struct Vec3 {
    T x = 0, y = 0, z = 0;
    constexpr Vec3() = default;
    NEON_CUDA_HOST_DEVICE constexpr Vec3(T a) : x(a), y(a), z(a) {}
    NEON_CUDA_HOST_DEVICE constexpr Vec3(T a, T b, T c) : x(a), y(b), z(c) {}
    template <typename U>
    NEON_CUDA_HOST_DEVICE constexpr Vec3<U> newType() const
    {
        return Vec3<U>(U(x), U(y), U(z));
    }
    NEON_CUDA_HOST_DEVICE constexpr Vec3 operator+(const Vec3& o) const { return Vec3(x + o.x, y + o.y, z + o.z); }
    NEON_CUDA_HOST_DEVICE constexpr Vec3 operator-(const Vec3& o) const { return Vec3(x - o.x, y - o.y, z - o.z); }
    NEON_CUDA_HOST_DEVICE constexpr Vec3 operator*(const Vec3& o) const { return Vec3(x * o.x, y * o.y, z * o.z); }
    NEON_CUDA_HOST_DEVICE constexpr Vec3 operator*(T s) const { return Vec3(x * s, y * s, z * s); }
    NEON_CUDA_HOST_DEVICE constexpr bool operator==(const Vec3& o) const { return x == o.x && y == o.y && z == o.z; }
    NEON_CUDA_HOST_DEVICE constexpr bool operator!=(const Vec3& o) const { return !(*this == o); }
    // component-wise "all less than" as Neon's vector comparison (vec3d_integer)
    NEON_CUDA_HOST_DEVICE constexpr bool operator<(const Vec3& o) const { return x < o.x && y < o.y && z < o.z; }
    NEON_CUDA_HOST_DEVICE constexpr T    rMul() const { return x * y * z; }
    template <typename U>
    NEON_CUDA_HOST_DEVICE constexpr U rMulTyped() const
    {
        return U(x) * U(y) * U(z);
    }
    NEON_CUDA_HOST_DEVICE T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    NEON_CUDA_HOST_DEVICE T  operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    // Neon's vectors also expose v[] (RunCavityTwoPop.cu:179)
    struct VView {
        const Vec3* p;
        NEON_CUDA_HOST_DEVICE T operator[](int i) const { return (*p)[i]; }
    };
    NEON_CUDA_HOST_DEVICE VView v_() const { return VView{this}; }
    std::string to_string() const
    {
        std::ostringstream s;
        s << "(" << +x << ", " << +y << ", " << +z << ")";
        return s.str();
    }
};
template <typename T>
inline std::ostream& operator<<(std::ostream& os, const Vec3<T>& v)
{
    return os << v.to_string();
}

using index_3d = Vec3<int32_t>;
using int32_3d = Vec3<int32_t>;
using uint32_3d = Vec3<uint32_t>;
using int8_3d = Vec3<int8_t>;
using int64_3d = Vec3<int64_t>;
using double_3d = Vec3<double>;
using float_3d = Vec3<float>;
template <typename T>
using Vec_3d = Vec3<T>;

// ------------------------------------------------------------------ enums (names of libNeonCore/libNeonSet)
enum class DataView { STANDARD = 0, INTERNAL = 1, BOUNDARY = 2 };
enum class Execution { device, host };
enum class Pattern { MAP, STENCIL, REDUCE };
enum class DataUse { HOST_DEVICE, COMPUTE, IO_COMPUTE, IO_POSTPROCESSING };
enum class MemoryLayout { structOfArrays, arrayOfStructs };
enum class Runtime { none, system, stream, openmp };
enum class computeMode_t { seq, par };

struct MemoryOptions {
    MemoryLayout order = MemoryLayout::structOfArrays;
    MemoryOptions() = default;
    void setOrder(MemoryLayout o) { order = o; }
};

namespace set {
enum class StencilSemantic { standard, streaming };
enum class TransferMode { put, get };
}  // namespace set

inline void init() {}

}  // namespace Neon
