// Test-infrastructure shim for the reference oracle build (serialization is a no-op).
#pragma once
