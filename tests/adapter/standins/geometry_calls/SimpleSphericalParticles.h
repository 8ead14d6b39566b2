// Stand-in for MegaMol's particle list (plugins/geometry_calls/include/geometry_calls/SimpleSphericalParticles.h:
// 27-64 enumerators, 371-589 accessors), for building the MegaMol adapter where the MegaMol tree is absent: the
// list's data pointers, strides, types, count, global radius and colour, with the reference's enumerator values.
#pragma once

#include <cstdint>

namespace megamol::geocalls {

class SimpleSphericalParticles {
public:
    enum VertexDataType { VERTDATA_NONE = 0, VERTDATA_FLOAT_XYZ = 1, VERTDATA_FLOAT_XYZR = 2, VERTDATA_SHORT_XYZ = 3,
                          VERTDATA_DOUBLE_XYZ = 4 };
    enum ColourDataType { COLDATA_NONE = 0, COLDATA_UINT8_RGB = 1, COLDATA_UINT8_RGBA = 2, COLDATA_FLOAT_RGB = 3,
                          COLDATA_FLOAT_RGBA = 4, COLDATA_FLOAT_I = 5, COLDATA_USHORT_RGBA = 6, COLDATA_DOUBLE_I = 7 };
    enum DirDataType { DIRDATA_NONE = 0, DIRDATA_FLOAT_XYZ = 1 };

    uint64_t GetCount() const { return count_; }
    void SetCount(uint64_t c) { count_ = c; }
    float GetGlobalRadius() const { return radius_; }
    void SetGlobalRadius(float r) { radius_ = r; }
    const unsigned char* GetGlobalColour() const { return colour_; }
    void SetGlobalColour(unsigned char r, unsigned char g, unsigned char b, unsigned char a = 255) {
        colour_[0] = r, colour_[1] = g, colour_[2] = b, colour_[3] = a;
    }

    VertexDataType GetVertexDataType() const { return vtype_; }
    const void* GetVertexData() const { return vdata_; }
    unsigned int GetVertexDataStride() const { return vstride_; }
    void SetVertexData(VertexDataType t, const void* p, unsigned int s = 0) {
        vtype_ = t, vdata_ = p, vstride_ = s;
    }

    ColourDataType GetColourDataType() const { return ctype_; }
    const void* GetColourData() const { return cdata_; }
    unsigned int GetColourDataStride() const { return cstride_; }
    void SetColourData(ColourDataType t, const void* p, unsigned int s = 0) {
        ctype_ = t, cdata_ = p, cstride_ = s;
    }
    void SetColourMapIndexValues(float lo, float hi) { cmin_ = lo, cmax_ = hi; }
    float GetMinColourIndexValue() const { return cmin_; }
    float GetMaxColourIndexValue() const { return cmax_; }

    DirDataType GetDirDataType() const { return dtype_; }
    const void* GetDirData() const { return ddata_; }
    unsigned int GetDirDataStride() const { return dstride_; }
    void SetDirData(DirDataType t, const void* p, unsigned int s = 0) {
        dtype_ = t, ddata_ = p, dstride_ = s;
    }

private:
    uint64_t count_ = 0;
    float radius_ = 0.5f;
    unsigned char colour_[4] = {255, 255, 255, 255};
    VertexDataType vtype_ = VERTDATA_NONE;
    const void* vdata_ = nullptr;
    unsigned int vstride_ = 0;
    ColourDataType ctype_ = COLDATA_NONE;
    const void* cdata_ = nullptr;
    unsigned int cstride_ = 0;
    float cmin_ = 0.0f, cmax_ = 1.0f;
    DirDataType dtype_ = DIRDATA_NONE;
    const void* ddata_ = nullptr;
    unsigned int dstride_ = 0;
};

}  // namespace megamol::geocalls
