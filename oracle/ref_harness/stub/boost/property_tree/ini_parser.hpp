// Stand-in for the one Boost facility the reference's tissue examples use
// (examples/TumorHeatEqnFDM/TumorHeatEqnFDM.hpp and examples/
// MRIDataPBHEqnFDM/MRIDataPBHEqnFDM.hpp read their physical constants with
// ptree::get<CT>("Parameters.NAME")).  Boost is not installed here; this
// header gives the reference-driver programs a ptree that holds numbers put
// by the program itself, so that those classes compile unmodified.  It is
// test infrastructure (checker builds only) and implements nothing else of
// Boost.PropertyTree.
#pragma once

#include <map>
#include <stdexcept>
#include <string>

namespace boost {
namespace property_tree {

class ptree {
public:
    template <class T>
    T get(const std::string& key) const {
        const auto it = values_.find(key);
        if (it == values_.end()) throw std::runtime_error("ptree stub: no value for " + key);
        return static_cast<T>(it->second);
    }
    void put(const std::string& key, double value) { values_[key] = value; }

private:
    std::map<std::string, double> values_;
};

}  // namespace property_tree
}  // namespace boost
