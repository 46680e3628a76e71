// Test-only empty stand-in: gsStaticBase.h includes its .hpp, which the reference tree does not
// ship as a header (its definitions are in the header itself).
#pragma once
