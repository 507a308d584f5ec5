// Minimal stand-in for the LS-DYNA keyword reader that the reference expects as
// a git submodule (lib/LSDynaReader, absent from the reference checkout).
// Only the members that Domain_d::CreateFromLSDyna reads are declared; this
// header exists solely so the reference CPU sources compile into the test
// oracle under oracle/_ref/. It contains no reader logic.
#ifndef WF_ORACLE_LSDYNA_STUB_H
#define WF_ORACLE_LSDYNA_STUB_H
#include <vector>
namespace LS_Dyna {
struct ls_node {
  int m_id = 0;
  double m_x[3] = {0.0, 0.0, 0.0};
};
struct ls_element {
  int id = 0;
  std::vector<int> node;
};
class lsdynaReader {
 public:
  std::vector<ls_node> m_node;
  std::vector<ls_element> m_elem;
  int m_elem_count = 0;
  lsdynaReader() {}
  explicit lsdynaReader(const char *) {}
};
}  // namespace LS_Dyna
#endif
