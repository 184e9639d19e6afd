// yaml_decl.h -- TEST INFRASTRUCTURE ONLY.
//
// The reference's plan-generator header (core/components/execution_plan_generator.h)
// names YAML::Node / YAML::LoadFile inside a constructor that the CPU oracle
// never calls.  These declarations only let that header compile; there are no
// definitions, so any call would fail to link.  yaml-cpp itself is not
// vendored in the reference and is not used by the oracle.
#pragma once
#include <string>

namespace YAML {
class Node {
 public:
  Node();
  template <class T>
  T as() const;
};
Node LoadFile(const std::string& path);
}  // namespace YAML
