// curvedSpaceSimDatabase.hpp - state persistence with the datasets of the reference's simpleModelDatabase
// (src/databases/simpleModelDatabase.cpp:9-158): per record the time, R3 positions, barycentric positions, face
// indices and optionally velocities, forces and types.  The reference stores them as extendable HDF5 datasets; HDF5 is
// not available to this build, so the records go to a flat little-endian binary file with a fixed record size
// (random access by record index):
//
//   header (24 bytes): char magic[8] = "CSSGDB01", int32 N, int32 flags (1 velocity, 2 force, 4 type), int64 reserved
//   record:            double time, double R3position[3N], double barycentricPosition[3N], int32 faceIndex[N],
//                      [double velocity[3N]], [double force[3N]], [int32 type[N]]
//
// curvedspacesim_gb300/database.py reads and writes the same layout.  valueVectorDatabase (below) does the same for
// the reference's value + vector records (vectorValueDatabase.cpp).
#ifndef CURVED_SPACE_SIM_DATABASE_HPP
#define CURVED_SPACE_SIM_DATABASE_HPP

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

namespace cssg {

struct fileMode {
    enum Enum { readonly, readwrite, replace };
};

class simpleModelDatabase {
public:
    simpleModelDatabase(int numberOfParticles, const std::string& fn, fileMode::Enum mode, bool saveVelocities = false,
                        bool saveTypes = false, bool saveForces = false)
        : N(numberOfParticles), filename(fn), mode_(mode), velocity(saveVelocities), type(saveTypes),
          force(saveForces)
    {
        if (mode == fileMode::replace) {
            write_header();
        } else {
            FILE* f = std::fopen(fn.c_str(), "rb");
            if (!f) {
                if (mode == fileMode::readonly) throw std::runtime_error("simpleModelDatabase: cannot open " + fn);
                write_header();
            } else {
                char magic[8];
                int32_t hn = 0, flags = 0;
                int64_t reserved = 0;
                bool ok = std::fread(magic, 1, 8, f) == 8 && std::fread(&hn, 4, 1, f) == 1 &&
                          std::fread(&flags, 4, 1, f) == 1 && std::fread(&reserved, 8, 1, f) == 1;
                std::fclose(f);
                if (!ok || std::memcmp(magic, "CSSGDB01", 8) != 0 || hn != N)
                    throw std::runtime_error("simpleModelDatabase: " + fn + " is not a database of " +
                                             std::to_string(N) + " particles");
                velocity = flags & 1;
                force = flags & 2;
                type = flags & 4;
            }
        }
    }

    //! bytes of one record
    size_t recordBytes() const
    {
        size_t b = 8 + 2 * 24 * (size_t)N + 4 * (size_t)N;
        if (velocity) b += 24 * (size_t)N;
        if (force) b += 24 * (size_t)N;
        if (type) b += 4 * (size_t)N;
        return b;
    }

    unsigned long currentNumberOfRecords() const
    {
        FILE* f = std::fopen(filename.c_str(), "rb");
        if (!f) return 0;
        std::fseek(f, 0, SEEK_END);
        long size = std::ftell(f);
        std::fclose(f);
        return size < 24 ? 0 : (unsigned long)((size - 24) / recordBytes());
    }

    //! simpleModelDatabase::writeState (:60-120): appends one record (record >= 0 is not supported, as in the reference)
    void writeState(const std::vector<double>& r3, const std::vector<double>& bary, const std::vector<int>& face,
                    const std::vector<double>& vel, const std::vector<double>& frc, const std::vector<int>& types,
                    double time, int record = -1)
    {
        if (record >= 0) throw std::runtime_error("overwriting specific records not implemented at the moment");
        if (mode_ == fileMode::readonly) throw std::runtime_error("simpleModelDatabase: opened read-only");
        FILE* f = std::fopen(filename.c_str(), "ab");
        if (!f) throw std::runtime_error("simpleModelDatabase: cannot append to " + filename);
        std::fwrite(&time, 8, 1, f);
        put(f, r3, 3 * (size_t)N);
        put(f, bary, 3 * (size_t)N);
        put(f, face, (size_t)N);
        if (velocity) put(f, vel, 3 * (size_t)N);
        if (force) put(f, frc, 3 * (size_t)N);
        if (type) put(f, types, (size_t)N);
        std::fclose(f);
    }

    //! simpleModelDatabase::readState (:122-158): the record's time, positions and the optional fields
    double readState(int rec, std::vector<double>& bary, std::vector<int>& face, std::vector<double>& vel,
                     std::vector<double>& frc, std::vector<int>& types, std::vector<double>* r3 = nullptr) const
    {
        FILE* f = std::fopen(filename.c_str(), "rb");
        if (!f) throw std::runtime_error("simpleModelDatabase: cannot open " + filename);
        if (rec < 0 || (unsigned long)rec >= currentNumberOfRecords()) {
            std::fclose(f);
            throw std::runtime_error("simpleModelDatabase: no record " + std::to_string(rec));
        }
        std::fseek(f, (long)(24 + recordBytes() * (size_t)rec), SEEK_SET);
        double time = 0;
        std::vector<double> r3v;
        bool ok = std::fread(&time, 8, 1, f) == 1 && get(f, r3v, 3 * (size_t)N) && get(f, bary, 3 * (size_t)N) &&
                  get(f, face, (size_t)N);
        if (ok && velocity) ok = get(f, vel, 3 * (size_t)N);
        if (ok && force) ok = get(f, frc, 3 * (size_t)N);
        if (ok && type) ok = get(f, types, (size_t)N);
        std::fclose(f);
        if (!ok) throw std::runtime_error("simpleModelDatabase: truncated record");
        if (r3) *r3 = r3v;
        return time;
    }

    int N;
    std::string filename;

private:
    void write_header()
    {
        FILE* f = std::fopen(filename.c_str(), "wb");
        if (!f) throw std::runtime_error("simpleModelDatabase: cannot create " + filename);
        int32_t n = N, flags = (velocity ? 1 : 0) | (force ? 2 : 0) | (type ? 4 : 0);
        int64_t reserved = 0;
        std::fwrite("CSSGDB01", 1, 8, f);
        std::fwrite(&n, 4, 1, f);
        std::fwrite(&flags, 4, 1, f);
        std::fwrite(&reserved, 8, 1, f);
        std::fclose(f);
    }
    template <typename T>
    static void put(FILE* f, const std::vector<T>& v, size_t count)
    {
        if (v.size() < count) throw std::runtime_error("simpleModelDatabase: array shorter than the record field");
        std::fwrite(v.data(), sizeof(T), count, f);
    }
    template <typename T>
    static bool get(FILE* f, std::vector<T>& v, size_t count)
    {
        v.resize(count);
        return std::fread(v.data(), sizeof(T), count, f) == count;
    }

    fileMode::Enum mode_;
    bool velocity, type, force;
};

//! valueVectorDatabase (src/databases/vectorValueDatabase.cpp:4-43): per record one double ("value") and a vector of
//! a fixed size ("vector"), both appended by writeState.  Flat little-endian layout like simpleModelDatabase:
//!
//!   header (24 bytes): char magic[8] = "CSSGVV01", int64 vectorSize, int64 reserved
//!   record:            double value, double vector[vectorSize]
class valueVectorDatabase {
public:
    valueVectorDatabase(const std::string& fn, unsigned long vectorSize, fileMode::Enum mode = fileMode::readonly)
        : filename(fn), maximumVectorSize(vectorSize), mode_(mode)
    {
        valueVector.resize(1);
        dataVector.resize(maximumVectorSize);
        FILE* f = std::fopen(fn.c_str(), "rb");
        if (mode == fileMode::replace || (mode == fileMode::readwrite && !f)) {
            if (f) std::fclose(f);
            write_header();
            return;
        }
        if (!f) throw std::runtime_error("valueVectorDatabase: cannot open " + fn);
        char magic[8];
        int64_t size = 0, reserved = 0;
        bool ok = std::fread(magic, 1, 8, f) == 8 && std::fread(&size, 8, 1, f) == 1 &&
                  std::fread(&reserved, 8, 1, f) == 1;
        std::fclose(f);
        if (!ok || std::memcmp(magic, "CSSGVV01", 8) != 0 || (unsigned long)size != maximumVectorSize)
            throw std::runtime_error("valueVectorDatabase: " + fn + " is not a database of vectors of size " +
                                     std::to_string(maximumVectorSize));
    }

    unsigned long currentNumberOfRecords() const
    {
        FILE* f = std::fopen(filename.c_str(), "rb");
        if (!f) return 0;
        std::fseek(f, 0, SEEK_END);
        long size = std::ftell(f);
        std::fclose(f);
        const size_t rec = 8 * (1 + maximumVectorSize);
        return size < 24 ? 0 : (unsigned long)((size - 24) / rec);
    }

    //! vectorValueDatabase.cpp:31-37: appends value and data (data must hold vectorSize entries)
    void writeState(double val, std::vector<double>& data)
    {
        if (mode_ == fileMode::readonly) throw std::runtime_error("valueVectorDatabase: opened read-only");
        if (data.size() < maximumVectorSize)
            throw std::runtime_error("valueVectorDatabase: vector shorter than the record");
        FILE* f = std::fopen(filename.c_str(), "ab");
        if (!f) throw std::runtime_error("valueVectorDatabase: cannot append to " + filename);
        std::fwrite(&val, 8, 1, f);
        std::fwrite(data.data(), 8, maximumVectorSize, f);
        std::fclose(f);
    }

    //! vectorValueDatabase.cpp:39-43: fills valueVector[0] and dataVector from record `record`
    void readState(int record)
    {
        if (record < 0 || (unsigned long)record >= currentNumberOfRecords())
            throw std::runtime_error("valueVectorDatabase: no record " + std::to_string(record));
        FILE* f = std::fopen(filename.c_str(), "rb");
        if (!f) throw std::runtime_error("valueVectorDatabase: cannot open " + filename);
        std::fseek(f, (long)(24 + 8 * (1 + maximumVectorSize) * (size_t)record), SEEK_SET);
        bool ok = std::fread(valueVector.data(), 8, 1, f) == 1 &&
                  std::fread(dataVector.data(), 8, maximumVectorSize, f) == maximumVectorSize;
        std::fclose(f);
        if (!ok) throw std::runtime_error("valueVectorDatabase: truncated record");
    }

    std::string filename;
    unsigned long maximumVectorSize;
    std::vector<double> valueVector, dataVector;

private:
    void write_header()
    {
        FILE* f = std::fopen(filename.c_str(), "wb");
        if (!f) throw std::runtime_error("valueVectorDatabase: cannot create " + filename);
        int64_t size = (int64_t)maximumVectorSize, reserved = 0;
        std::fwrite("CSSGVV01", 1, 8, f);
        std::fwrite(&size, 8, 1, f);
        std::fwrite(&reserved, 8, 1, f);
        std::fclose(f);
    }
    fileMode::Enum mode_;
};

}  // namespace cssg

#endif
