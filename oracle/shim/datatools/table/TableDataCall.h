// Minimal stand-in for MegaMol's TableDataCall (plugins/datatools/include/datatools/table/
// TableDataCall.h), oracle build only: the column-info setters and Set() that ParticlesToDensity uses.
#pragma once

#include <string>

#include "mmcore/Call.h"

namespace megamol::datatools::table {

class TableDataCall : public core::Call {
public:
    enum class ColumnType { CATEGORICAL, QUANTITATIVE };

    class ColumnInfo {
    public:
        ColumnInfo& SetName(const std::string& n) {
            name_ = n;
            return *this;
        }
        ColumnInfo& SetType(ColumnType t) {
            type_ = t;
            return *this;
        }
        ColumnInfo& SetMinimumValue(float v) {
            min_ = v;
            return *this;
        }
        ColumnInfo& SetMaximumValue(float v) {
            max_ = v;
            return *this;
        }
        const std::string& Name() const {
            return name_;
        }
        float MinimumValue() const {
            return min_;
        }
        float MaximumValue() const {
            return max_;
        }

    private:
        std::string name_;
        ColumnType type_ = ColumnType::QUANTITATIVE;
        float min_ = 0.0f, max_ = 0.0f;
    };

    static const char* ClassName() {
        return "TableDataCall";
    }
    static const char* FunctionName(unsigned int idx) {
        return idx == 0 ? "GetData" : "GetHash";
    }

    void Set(size_t cols, size_t rows, const ColumnInfo* infos, const float* data) {
        cols_ = cols;
        rows_ = rows;
        infos_ = infos;
        data_ = data;
    }
    void SetDataHash(size_t h) {
        hash_ = h;
    }
    size_t GetColumnsCount() const {
        return cols_;
    }
    size_t GetRowsCount() const {
        return rows_;
    }
    const ColumnInfo* GetColumnsInfos() const {
        return infos_;
    }
    const float* GetData() const {
        return data_;
    }
    void SetUnlocker(void*, bool = true) {}
    void SetFrameCount(unsigned int n) {
        frames_ = n;
    }

private:
    size_t cols_ = 0, rows_ = 0, hash_ = 0;
    unsigned int frames_ = 1;
    const ColumnInfo* infos_ = nullptr;
    const float* data_ = nullptr;
};

} // namespace megamol::datatools::table
