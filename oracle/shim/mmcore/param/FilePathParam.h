// Minimal stand-in for MegaMol's FilePathParam (core/include/mmcore/param/FilePathParam.h), oracle build
// only: a parameter holding a std::filesystem::path.
#pragma once

#include <filesystem>
#include <string>
#include <vector>

#include "mmcore/param/ParamSlot.h"

namespace megamol::core::param {

class FilePathParam : public AbstractParam {
public:
    enum FilePathFlags_ : int {
        Flag_File = 1 << 0,
        Flag_Directory = 1 << 1,
        Flag_NoExistenceCheck = 1 << 2,
        Flag_RestrictExtension = 1 << 3,
        Flag_File_ToBeCreated = Flag_File | Flag_NoExistenceCheck,
        Flag_File_RestrictExtension = Flag_File | Flag_RestrictExtension,
    };
    explicit FilePathParam(const std::string& v, int = 0, const std::vector<std::string>& = {}) : value_(v) {}
    const std::filesystem::path& Value() const {
        return value_;
    }
    void SetValue(const std::filesystem::path& v, bool = true) {
        value_ = v;
        dirty = true;
    }

private:
    std::filesystem::path value_;
};

} // namespace megamol::core::param
