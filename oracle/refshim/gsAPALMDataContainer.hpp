// Test-only stand-in: the reference tree ships gsAPALMDataContainer.h with every member
// defined inline and no .hpp; this empty file completes its include.
#pragma once
