// oracle/shim/tinyxml2.h -- TEST INFRASTRUCTURE ONLY.
// The reference's XMLBIFParser.h includes tinyxml2 (not vendored here).  The reference
// driver only loads plain BIF files (CustomNetwork::LoadBIFFile), so these declarations
// just let CustomNetwork.cpp compile; xmlbif_stub.cpp aborts if the XML path is ever used.
#pragma once
namespace tinyxml2 {
class XMLElement {
public:
    const char *GetText() const;
};
class XMLDocument {};
}  // namespace tinyxml2
