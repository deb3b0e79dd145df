// oracle/shim/xmlbif_stub.cpp -- TEST INFRASTRUCTURE ONLY.
// Link stubs for the XML-BIF entry points that CustomNetwork.cpp references; the reference
// driver never calls them (it loads plain BIF files), so each one aborts.
#include <cstdio>
#include <cstdlib>
#include "fastpgm/XMLBIFParser.h"

const char *tinyxml2::XMLElement::GetText() const {
    fprintf(stderr, "XML-BIF is not available in the reference driver\n");
    abort();
}
XMLBIFParser::XMLBIFParser(string &) {
    fprintf(stderr, "XML-BIF is not available in the reference driver\n");
    abort();
}
vector<Node *> XMLBIFParser::GetConnectedNodes(int) {
    fprintf(stderr, "XML-BIF is not available in the reference driver\n");
    abort();
}
