/*
 * Model descriptors of the GB300 backend, for the per-model processor
 * factory ac::core::Processor::create<Processor::CUDA, Model>(device, model).
 *
 * The class names and their Variant enumerators are the reference's
 * (core/include/AC/Core/Model/ACNet.hpp:18-116, ARNet.hpp:16-72,
 * ArtCNN.hpp:16-60, FSRCNNX.hpp:16-70), so code that selects a model the
 * reference's way compiles unchanged.  Here a model only names a network and
 * its variant: the processor owns the parameters, device-resident and packed
 * for its kernels, and the reference's per-layer parameter accessors are not
 * part of this interface.  ARNet runs its exact topology with seeded
 * synthetic parameters (the reference's trained ARNet parameters are not in
 * its source tree).
 */
#ifndef AC_GB300_CXX_MODEL_HPP
#define AC_GB300_CXX_MODEL_HPP

namespace ac::core::model
{
    class ACNetLegacy
    {
    public:
        enum class Variant
        {
            GAN,
            HDN0,
            HDN1,
            HDN2,
            HDN3
        };
        ACNetLegacy(Variant v) noexcept : v_(v) {}
        Variant variant() const noexcept { return v_; }
        int blocks() const noexcept { return 8; }

    private:
        Variant v_;
    };

    template<int F>
    class ACNet
    {
        static_assert(F == 8, "ACNet has 8 feature channels");

    public:
        enum class Variant
        {
            B4_NORMAL, B4_HDN, B4_BOX, B4_BOX_HDN,
            B8_NORMAL, B8_HDN, B8_BOX, B8_BOX_HDN,
            B18_NORMAL, B18_HDN, B18_BOX, B18_BOX_HDN
        };
        ACNet(Variant v) noexcept : v_(v) {}
        Variant variant() const noexcept { return v_; }
        int blocks() const noexcept
        {
            const int g = static_cast<int>(v_) / 4;
            return g == 0 ? 4 : (g == 1 ? 8 : 18);
        }

    private:
        Variant v_;
    };

    template<int F>
    class ARNet
    {
        static_assert(F == 8, "ARNet has 8 feature channels");

    public:
        enum class Variant
        {
            B8_NORMAL, B8_HDN, B8_BOX, B8_BOX_HDN,
            B16_NORMAL, B16_HDN, B16_BOX, B16_BOX_HDN,
            B32_NORMAL, B32_HDN, B32_BOX, B32_BOX_HDN,
            B64_NORMAL, B64_HDN, B64_BOX, B64_BOX_HDN
        };
        ARNet(Variant v) noexcept : v_(v) {}
        Variant variant() const noexcept { return v_; }
        int blocks() const noexcept { return 8 << (static_cast<int>(v_) / 4); }

    private:
        Variant v_;
    };

    template<int F>
    class ArtCNN
    {
        static_assert(F == 16 || F == 32, "ArtCNN has 16 or 32 feature channels");

    public:
        enum class Variant
        {
            C4_NORMAL, C4_DN, C4_DS
        };
        ArtCNN(Variant v) noexcept : v_(v) {}
        Variant variant() const noexcept { return v_; }
        int blocks() const noexcept { return 4; }

    private:
        Variant v_;
    };

    template<int F>
    class FSRCNNX
    {
        static_assert(F == 8 || F == 16, "FSRCNNX has 8 or 16 feature channels");

    public:
        enum class Variant
        {
            B4_NORMAL, B4_DISTORT_PLUS
        };
        FSRCNNX(Variant v) noexcept : v_(v) {}
        Variant variant() const noexcept { return v_; }
        int blocks() const noexcept { return 4; }

    private:
        Variant v_;
    };
}

#endif
